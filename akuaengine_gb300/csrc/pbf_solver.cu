// Host side of the GB300 PBF step: device memory, the per-step launch sequence, CUDA-graph
// capture and the C ABI declared in include/akua_pbf.h.
//
// One handle = one particle set on one device.  A step is [params] [import + sort keys, or the
// keys alone when the state stayed on the device] and then the captured body: radix sort by
// (hash, previous reference rank) beside radix sort by Morton cell -> gather into the new internal
// order -> bucket table -> neighbour walk (+ iteration 1 density/lambda) -> (delta+correct,
// density+lambda) x iterations -> delta+update+damping -> vorticity -> confinement -> XSPH (which
// also empties the bucket table) -> export in reference order.  Nothing on this path copies to
// the host or synchronises; the reference instead synchronises after every kernel and moves the
// neighbour lists through host memory four times per step (PBFSolver.h:23-24,
// NeighbourSearchCUDA.cu:151-154, 182-183, ConstraintSolverCUDA.cu:195-198,
// IntegrationCUDA.cu:269-272).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "akua_pbf.h"
#include "mlp_handle.h"
#include "pbf_kernels.cuh"
#include "pbf_learned.cuh"
#include "radix_sort.cuh"

using akua::StepParams;

struct akua_pbf {
    int device = 0;
    int n = 0;
    akua_pbf_config cfg{};
    akua_lambda_corr_params corr{};
    uint32_t table_size = 0;
    uint32_t table_alloc = 0;
    float restitution = 0.0f;
    float friction = 0.95f;
    uint32_t options = 0;
    cudaStream_t stream = nullptr;          // caller's stream (nullptr = legacy default stream)
    cudaStream_t capture_stream = nullptr;  // private stream used only for graph capture
    char* attached = nullptr;
    size_t stride = 0;
    bool state_valid = false;  // device state holds the particles (resident mode)
    bool stepped = false;      // the reference-order tables describe the current state

    StepParams* d_params = nullptr;
    // state, internal order
    float4 *x4 = nullptr, *v4 = nullptr, *col4 = nullptr;
    float* size = nullptr;
    uint32_t* rref = nullptr;
    float *rho = nullptr, *lam = nullptr;
    float4* dp4 = nullptr;
    // gathered copies and per-step arrays
    float4 *x4g = nullptr, *col4g = nullptr, *ps0 = nullptr, *ps1 = nullptr;
    float4 *vstar4 = nullptr, *om4 = nullptr, *xv8 = nullptr, *dpg = nullptr, *xref = nullptr;
    float *sizeg = nullptr, *rhog = nullptr, *lamg = nullptr;
    uint32_t *rrefg = nullptr, *rank_of_import = nullptr, *r2i = nullptr, *order = nullptr;
    // sorts: reference order (A) and Morton order (B)
    uint32_t *ka0 = nullptr, *va0 = nullptr, *ka1 = nullptr, *va1 = nullptr;
    uint32_t *kb0 = nullptr, *vb0 = nullptr, *kb1 = nullptr, *vb1 = nullptr;
    uint32_t* sort_scratch = nullptr;
    uint32_t* sort_scratch_b = nullptr;  // the Morton sort's, which runs beside the hash sort
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    uint2* table = nullptr;
    uint32_t *nbr = nullptr, *cnt = nullptr, *flags = nullptr;
    float4* psl = nullptr;          // (x*, lambda) of the current iteration, for uniform masses
    akua::SdfShape* shapes = nullptr;  // SDF obstacles (device), AKUA_SDF_MAX_SHAPES
    int num_shapes = 0;
    float sdf_min_dist = 0.025f, sdf_stiffness = 0.5f;
    uint32_t* mass_bits = nullptr;  // {another mass seen, record 0's mass bits} of this step
    char* staging = nullptr;
    size_t staging_bytes = 0;

    akua::radix::Plan plan_ref, plan_sp;
    int sp_bits = 0;
    uint32_t *kr = nullptr, *refperm = nullptr, *spperm = nullptr;  // sort results (set at enqueue)

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool graph_ok = false;
    uint32_t graph_options = 0;
    const char* graph_aos = nullptr;
    size_t graph_stride = 0;
    int graph_sp_bits = -1;
    int graph_captures = 0;
    int body_launches = 0;

    // learned warm start (allocated on first use): features, predicted velocity (.w = density),
    // the step's accumulated lambda, the previous step's (internal order) and the export copy
    // (reference order, read back at import)
    akua_mlp* warm = nullptr;
    bool track = false;  // accumulate lambda and compute features every step
    float* cap_feat = nullptr;
    float* cap_target = nullptr;
    float *feat = nullptr, *lacc = nullptr, *lprev = nullptr, *lacc_ref = nullptr;
    float* speed = nullptr;
    uint32_t* err_max = nullptr;
    double* err_sum = nullptr;
    int graph_learn = 0;

    // batches of independent scenes (akua_pbf_create_batch); empty for a single scene
    std::vector<akua_scene_desc> scenes;
    std::vector<uint32_t> scene_first;  // first particle of each scene
    uint16_t* scene_of = nullptr;       // device: the scene of every particle
    int scene_bits = 0;                 // bits of the scene index in the Morton sort key

    // block sizes of the neighbour-pair kernels (akua_pbf_set_pair_blocks / akua_pbf_autotune)
    int pair_block[AKUA_PBF_PAIR_KERNELS] = {128, 128, 128, 128, 128, 128};
    // the walk's tile shape (akua_pbf_set_search_shape / akua_pbf_autotune)
    int search_block = akua::kSearchBlock;
    int search_stage = akua::kListStage;

    int64_t steps = 0;
    uint64_t device_bytes = 0;

    // profiling (akua_pbf_profile_begin/end): one event after every kernel of a step
    bool prof_active = false;
    int prof_steps_left = 0;
    std::vector<cudaEvent_t> prof_events;
    std::vector<const char*> prof_names;  // nullptr marks the start of a step
    size_t prof_next = 0;
};

namespace akua::mlp {
int enqueue_forward(const akua_mlp* m, const float* feat, int n, float* out, float* out2,
                    float* out4, cudaStream_t st);
}

namespace {

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return AKUA_OK;
    if (e == cudaErrorMemoryAllocation) return AKUA_ERR_OUT_OF_MEMORY;
    return AKUA_ERR_CUDA;
}

template <class T>
cudaError_t dalloc(akua_pbf* s, T** p, size_t count) {
    const size_t bytes = count * sizeof(T);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), bytes > 0 ? bytes : sizeof(T));
    if (e == cudaSuccess) s->device_bytes += bytes;
    return e;
}

void free_all(akua_pbf* s) {
    void* ptrs[] = {s->d_params, s->x4, s->v4, s->col4, s->size, s->rref, s->rho, s->lam, s->dp4,
                    s->x4g, s->col4g, s->ps0, s->ps1, s->vstar4, s->om4, s->xv8, s->dpg, s->xref,
                    s->sizeg, s->rhog, s->lamg, s->rrefg, s->rank_of_import, s->r2i, s->order,
                    s->ka0, s->va0, s->ka1, s->va1, s->kb0, s->vb0, s->kb1, s->vb1,
                    s->sort_scratch, s->sort_scratch_b, s->table, s->nbr, s->cnt, s->flags,
                    s->staging,
                    s->feat, s->lacc, s->lprev, s->lacc_ref, s->speed, s->err_max, s->err_sum,
                    s->scene_of, s->psl, s->mass_bits, s->shapes};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    if (s->capture_stream) cudaStreamDestroy(s->capture_stream);
    if (s->side_stream) cudaStreamDestroy(s->side_stream);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    for (cudaEvent_t ev : s->prof_events) cudaEventDestroy(ev);
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

bool finite3(const float* v) {
    return v && std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]);
}

// Bits per axis of the Morton key for a box, and the lowest cell it counts from.
int morton_bits(const akua_pbf* s, const float* bmin, const float* bmax, int origin[3]) {
    const double cell = (double)s->cfg.spatialHashCellSize;
    double extent = 0.0;
    for (int a = 0; a < 3; ++a) {
        origin[a] = (int)std::floor((double)bmin[a] / cell) - 1;
        extent = std::max(extent, ((double)bmax[a] - (double)bmin[a]) / cell + 3.0);
    }
    int bits = 1;
    while (bits < 10 && (double)(1 << bits) < extent) ++bits;
    return bits;
}


// Kernel constants, evaluated on the host in the order the device and the host restatement use.
// Host code is compiled with -ffp-contract=off.
StepParams make_params(const akua_pbf* s, float dt, const float* bmin, const float* bmax) {
    StepParams p{};
    const float h = s->cfg.smoothRadius;
    p.h = h;
    p.h2 = h * h;
    const double pi_ref = (double)3.14f;  // SmoothingKernelsCUDA.h:20,27 write pi as 3.14f
    const double hd = (double)h;
    const double h2 = hd * hd, h3 = h2 * hd, h6 = h3 * h3, h9 = h6 * h3;
    p.kp = (float)(315.0 / (64.0 * pi_ref * h9));
    p.ks = (float)(-(45.0 / (pi_ref * h6)));
    {
        const float d = p.h2 - 0.0f;
        p.w0 = p.kp * ((d * d) * d);
    }
    p.inv_rho0 = 1.0f / s->cfg.restDensity;
    p.relaxation = s->cfg.relaxation;
    {
        const float dq2 = s->corr.delta_q * s->corr.delta_q;
        const float d = p.h2 - dq2;
        p.wdq = dq2 > p.h2 ? 0.0f : p.kp * ((d * d) * d);
        p.inv_wdq = 1.0f / p.wdq;
    }
    p.neg_k = -s->corr.k;
    p.corr_n = s->corr.n;
    const float nf = s->corr.n;
    p.corr_n_int = (std::floor(nf) == nf && nf >= 0.0f && nf <= 64.0f) ? (int32_t)nf : -1;
    p.hash_cell = h;  // the reference hashes with the smoothing radius (NeighbourSearchCUDA.cu:163)
    p.search_cell = s->cfg.spatialHashCellSize;
    p.vort_eps = s->cfg.vorticityEpsilon;
    p.visc = s->cfg.viscosity;
    p.dt = dt;
    for (int a = 0; a < 3; ++a) {
        p.gravity[a] = s->cfg.gravity[a];
        p.box_min[a] = bmin[a];
        p.box_max[a] = bmax[a];
    }
    p.neg_restitution = -s->restitution;
    p.keep = 1.0f - s->friction;
    p.n = s->n;
    p.cap = s->cfg.maxNeighbours;
    p.table_size = s->table_size;
    p.table_magic = UINT64_MAX / (uint64_t)s->table_size + 1u;
    p.sp_bits = morton_bits(s, bmin, bmax, p.sp_origin);
    p.shapes = s->shapes;
    p.num_shapes = s->num_shapes;
    p.sdf_min_dist = s->sdf_min_dist;
    p.sdf_stiffness = s->sdf_stiffness;
    return p;
}

// Parameters of every scene of a batch for one step.  The Morton keys of all scenes share one
// bit count per axis (the largest any box needs, limited so that the scene index fits above
// them in 32 bits; cells beyond it are clamped, which only costs locality).
std::vector<StepParams> make_batch_params(const akua_pbf* s, float dt) {
    const int ns = (int)s->scenes.size();
    std::vector<StepParams> out(ns);
    int bits = 1;
    std::vector<int> origin(3 * ns);
    for (int k = 0; k < ns; ++k)
        bits = std::max(bits, morton_bits(s, s->scenes[k].boxMin, s->scenes[k].boxMax,
                                          &origin[3 * k]));
    bits = std::min(bits, (32 - s->scene_bits) / 3);
    for (int k = 0; k < ns; ++k) {
        const akua_scene_desc& d = s->scenes[k];
        StepParams p = make_params(s, dt, d.boxMin, d.boxMax);
        for (int a = 0; a < 3; ++a) {
            p.gravity[a] = d.gravity[a];
            p.sp_origin[a] = origin[3 * k + a];
        }
        p.sp_bits = bits;
        // PBFSolver.cpp:15 per scene: maxNeighbours * N_s buckets, after the earlier scenes'
        p.table_size = (uint32_t)(s->cfg.maxNeighbours * d.numParticles);
        p.table_magic = UINT64_MAX / (uint64_t)p.table_size + 1u;
        p.table_offset = (uint32_t)s->cfg.maxNeighbours * s->scene_first[k];
        p.scene = k;
        p.scene_of = s->scene_of;
        out[k] = p;
    }
    return out;
}

inline int grid_for(int n, int block) { return (n + block - 1) / block; }

// 0: plain step; 1: features and accumulated lambda are tracked (training capture); 2: and the
// network's prediction replaces iteration 1's lambda.
int learn_mode(const akua_pbf* s) { return s->warm ? 2 : ((s->track || s->cap_feat) ? 1 : 0); }

cudaError_t ensure_learn_buffers(akua_pbf* s) {
    if (s->feat) return cudaSuccess;
    const int n = s->n;
    cudaError_t e = dalloc(s, &s->feat, (size_t)8 * n);
    if (e == cudaSuccess) e = dalloc(s, &s->lacc, n);
    if (e == cudaSuccess) e = dalloc(s, &s->lprev, n);
    if (e == cudaSuccess) e = dalloc(s, &s->lacc_ref, n);
    if (e == cudaSuccess) e = dalloc(s, &s->speed, n);
    if (e == cudaSuccess) e = dalloc(s, &s->err_max, 1);
    if (e == cudaSuccess) e = dalloc(s, &s->err_sum, 1);
    if (e == cudaSuccess) e = cudaMemset(s->lacc, 0, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMemset(s->lacc_ref, 0, sizeof(float) * n);
    return e;
}

// Counts launches and, while profiling (never during capture), records an event after each.
struct Marker {
    akua_pbf* s;
    cudaStream_t st;
    bool record;
    int launches = 0;
    void operator()(const char* name) {
        ++launches;
        if (record && s->prof_next < s->prof_events.size()) {
            cudaEventRecord(s->prof_events[s->prof_next], st);
            s->prof_names[s->prof_next] = name;
            ++s->prof_next;
        }
    }
};

// The walk at one tile shape (BLOCK threads, STAGE staged list entries per particle).
template <bool EXACT, int BLOCK, int STAGE>
void launch_search_shape(akua_pbf* s, cudaStream_t st, int density, float* feat) {
    akua::k_search<EXACT, BLOCK, STAGE><<<grid_for(s->n, BLOCK), BLOCK,
                                          akua::search_smem(BLOCK, STAGE), st>>>(
        s->d_params, s->ps0, s->xref, s->table, s->r2i, s->nbr, s->cnt, s->rho, s->lam,
        s->flags, density, s->speed, s->lprev, s->lacc, feat, s->psl);
}

template <bool EXACT>
void launch_search(akua_pbf* s, cudaStream_t st, int density, float* feat) {
    const int b = s->search_block, g = s->search_stage;
    if (g == 48) {  // 64 or 128 threads (256 x 48 entries would exceed 48 KB of shared memory)
        if (b == 64) launch_search_shape<EXACT, 64, 48>(s, st, density, feat);
        else launch_search_shape<EXACT, 128, 48>(s, st, density, feat);
    } else if (g == 16) {
        if (b == 64) launch_search_shape<EXACT, 64, 16>(s, st, density, feat);
        else if (b == 256) launch_search_shape<EXACT, 256, 16>(s, st, density, feat);
        else launch_search_shape<EXACT, 128, 16>(s, st, density, feat);
    } else {
        if (b == 64) launch_search_shape<EXACT, 64, 32>(s, st, density, feat);
        else if (b == 256) launch_search_shape<EXACT, 256, 32>(s, st, density, feat);
        else launch_search_shape<EXACT, 128, 32>(s, st, density, feat);
    }
}

template <bool EXACT>
void enqueue_pairs(akua_pbf* s, cudaStream_t st, Marker& mark) {
    const int n = s->n;
    const int* pb = s->pair_block;  // per kernel: density, delta, last delta, vort., conf., XSPH
    auto gp = [&](int k) { return grid_for(n, pb[k]); };
    const int iters = s->cfg.solverIterations;
    float4* ps[2] = {s->ps0, s->ps1};
    const uint4* nbr4 = reinterpret_cast<const uint4*>(s->nbr);
    const int learn = learn_mode(s);
    launch_search<EXACT>(s, st, iters > 0 ? 1 : 0, learn ? s->feat : nullptr);
    mark("k_search");
    if (learn == 2) {
        akua::mlp::enqueue_forward(s->warm, s->feat, n, s->lam, s->lacc, &s->psl->w, st);
        mark("k_mlp_forward");
    }
    for (int it = 0; it < iters; ++it) {
        float4* cur = ps[it & 1];
        float4* nxt = ps[(it + 1) & 1];
        if (it > 0) {
            akua::k_density_lambda<EXACT><<<gp(0), pb[0], 0, st>>>(
                s->d_params, cur, nbr4, s->cnt, s->rho, s->lam,
                learn == 1 ? s->lacc : nullptr, s->psl);  // warm: the network's estimate is the sum
            mark("k_density_lambda");
        }
        if (it + 1 < iters) {
            akua::k_delta_correct<EXACT><<<gp(1), pb[1], 0, st>>>(
                s->d_params, cur, s->lam, nbr4, s->cnt, nxt, s->dp4, s->psl, s->mass_bits);
            mark("k_delta_correct");
        } else {
            akua::k_delta_final<EXACT><<<gp(2), pb[2], 0, st>>>(
                s->d_params, cur, s->lam, nbr4, s->cnt, s->x4g, s->x4, s->v4, s->vstar4, s->dp4,
                s->col4g, s->sizeg, s->col4, s->size, s->rrefg, s->rref, s->rhog, s->lamg, s->dpg,
                s->rho, nullptr, 1, s->psl, s->mass_bits, s->xv8);  // lam_out: zero iterations only
            mark("k_delta_final");
        }
    }
    if (iters == 0) {
        akua::k_delta_final<EXACT><<<gp(2), pb[2], 0, st>>>(
            s->d_params, s->ps0, nullptr, nbr4, s->cnt, s->x4g, s->x4, s->v4, s->vstar4, s->dp4,
            s->col4g, s->sizeg, s->col4, s->size, s->rrefg, s->rref, s->rhog, s->lamg, s->dpg,
            s->rho, s->lam, 0, s->psl, s->mass_bits, s->xv8);  // no delta: lambda is not read
        mark("k_delta_final");
    }
    // psl is free after the last delta: it carries (x, |omega|) to confinement
    akua::k_vorticity<EXACT><<<gp(3), pb[3], 0, st>>>(s->d_params, s->x4, s->v4, s->xv8, nbr4,
                                                      s->cnt, s->om4, s->psl);
    mark("k_vorticity");
    akua::k_confine<EXACT><<<gp(4), pb[4], 0, st>>>(s->d_params, s->x4, s->v4, s->om4,
                                                    s->rho, nbr4, s->cnt, s->xv8, s->psl,
                                                    s->mass_bits);
    mark("k_confine");
    akua::k_xsph<<<gp(5), pb[5], 0, st>>>(s->d_params, s->xv8, nbr4, s->cnt, s->v4,
                                          s->kr, s->table);
    mark("k_xsph");
}

// Everything of a step after the parameter upload and the import: the captured body.
void enqueue_body(akua_pbf* s, cudaStream_t st, const char* aos, size_t stride, bool record) {
    const int n = s->n;
    const int ge = grid_for(n, akua::kElemBlock);
    Marker mark{s, st, record};
    const bool carry = s->cfg.solverIterations == 0;
    uint32_t* dummy = nullptr;
    // The two sorts are independent: reference order, stable by (hash, previous reference rank),
    // and internal order, stable by Morton cell over the previous reference order (payload: import
    // index).  Outside profiling the second runs on a side stream, a parallel branch of the graph.
    const bool fork = !record;
    cudaStream_t sb = st;
    Marker mark_b{s, st, record};
    if (fork) {
        cudaEventRecord(s->ev_fork, st);
        cudaStreamWaitEvent(s->side_stream, s->ev_fork, 0);
        sb = s->side_stream;
        mark_b = Marker{s, sb, false};
    }
    akua::radix::sort_pairs(sb, s->plan_sp, s->kb0, s->vb0, s->kb1, s->vb1, false,
                            s->sort_scratch_b, n, &dummy, &s->spperm, fork ? mark_b : mark);
    if (fork) cudaEventRecord(s->ev_join, sb);
    // the last pass also writes each import slot's reference rank (the inverse permutation)
    akua::radix::sort_pairs(st, s->plan_ref, s->ka0, s->va0, s->ka1, s->va1, false,
                            s->sort_scratch, n, &s->kr, &s->refperm, mark, s->rank_of_import);
    if (fork) {
        cudaStreamWaitEvent(st, s->ev_join, 0);
        mark.launches += mark_b.launches;
    }
    cudaMemsetAsync(s->mass_bits, 0, sizeof(uint32_t), st);  // "another mass seen" flag
    akua::k_gather<<<ge, akua::kElemBlock, 0, st>>>(
        s->d_params, s->spperm, s->rank_of_import, s->x4, s->v4, s->col4, s->size, s->rref, s->x4g,
        s->col4g, s->sizeg, s->ps0, s->r2i, s->rrefg, s->xref, s->order, s->rho, s->lam, s->dp4,
        s->rhog, s->lamg, s->dpg, carry ? 1 : 0, s->lacc, s->lprev,
        learn_mode(s) ? s->speed : nullptr, s->mass_bits);
    mark("k_gather");
    akua::k_table_build<<<ge, akua::kElemBlock, 0, st>>>(s->d_params, s->kr, s->r2i, s->table);
    mark("k_table_build");
    if (s->options & AKUA_PBF_OPT_EXACT_MATH) enqueue_pairs<true>(s, st, mark);
    else enqueue_pairs<false>(s, st, mark);
    if (aos) {
        akua::k_export<<<grid_for(n, akua::kIoBlock), akua::kIoBlock, 0, st>>>(
            s->d_params, const_cast<char*>(aos), stride, n, s->r2i, s->kr, s->x4, s->v4, s->vstar4, s->dp4,
            s->om4, s->rho, s->lam, s->col4, s->size, s->lacc,
            learn_mode(s) ? s->lacc_ref : nullptr);
        mark("k_export");
    }
    s->body_launches = mark.launches;
}

void invalidate_graph(akua_pbf* s) {
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
    s->graph_ok = false;
}

void update_plans(akua_pbf* s, int sp_bits) {
    s->plan_ref = akua::radix::make_plan(akua::radix::bits_for(s->table_size));
    s->sp_bits = sp_bits;
    s->plan_sp = akua::radix::make_plan(3 * sp_bits + s->scene_bits);
}

int ensure_graph(akua_pbf* s, const char* aos, size_t stride) {
    if (s->graph_ok && s->graph_options == s->options && s->graph_aos == aos &&
        s->graph_stride == stride && s->graph_sp_bits == s->sp_bits &&
        s->graph_learn == learn_mode(s))
        return AKUA_OK;
    invalidate_graph(s);
    cudaError_t e = cudaStreamBeginCapture(s->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e);
    enqueue_body(s, s->capture_stream, aos, stride, false);
    e = cudaStreamEndCapture(s->capture_stream, &s->graph);
    if (e != cudaSuccess) {
        s->graph = nullptr;
        return cuda_status(e);
    }
    e = cudaGraphInstantiate(&s->exec, s->graph, 0);
    if (e != cudaSuccess) {
        s->exec = nullptr;
        return cuda_status(e);
    }
    s->graph_ok = true;
    s->graph_options = s->options;
    s->graph_aos = aos;
    s->graph_stride = stride;
    s->graph_sp_bits = s->sp_bits;
    s->graph_learn = learn_mode(s);
    ++s->graph_captures;
    return AKUA_OK;
}

int do_step(akua_pbf* s, const char* aos, size_t stride, bool force_import, float dt,
            const float* bmin, const float* bmax) {
    const bool batch = !s->scenes.empty();
    if (!(std::isfinite(dt) && dt > 0.0f) || (!batch && (!finite3(bmin) || !finite3(bmax))))
        return AKUA_ERR_INVALID_ARGUMENT;
    cudaGetLastError();  // clear a stale error of an unrelated call
    const std::vector<StepParams> ps =
        batch ? make_batch_params(s, dt) : std::vector<StepParams>{make_params(s, dt, bmin, bmax)};
    const StepParams& p = ps[0];
    if (p.sp_bits != s->sp_bits) update_plans(s, p.sp_bits);
    cudaStream_t st = s->stream;
    const bool prof = s->prof_active && s->prof_steps_left > 0;
    Marker mark{s, st, prof};
    if (prof) {
        --s->prof_steps_left;
        if (s->prof_next < s->prof_events.size()) {  // step start
            cudaEventRecord(s->prof_events[s->prof_next], st);
            s->prof_names[s->prof_next++] = nullptr;
        }
    }
    if (!batch) {
        akua::k_set_params<<<1, 32, 0, st>>>(p, s->d_params);
    } else {
        for (size_t k0 = 0; k0 < ps.size(); k0 += akua::kParamChunk) {
            akua::ParamChunk c;
            c.count = (int)std::min(ps.size() - k0, (size_t)akua::kParamChunk);
            for (int k = 0; k < c.count; ++k) c.p[k] = ps[k0 + k];
            akua::k_set_params_chunk<<<1, akua::kParamChunk, 0, st>>>(c, s->d_params + k0);
        }
    }
    mark("k_set_params");
    const bool import = force_import || !(s->options & AKUA_PBF_OPT_RESIDENT) || !s->state_valid;
    if (import) {
        akua::k_import<<<grid_for(s->n, akua::kIoBlock), akua::kIoBlock, 0, st>>>(
            s->d_params, aos, stride, s->n, s->x4, s->v4, s->col4, s->size, s->rref, s->rho,
            s->lam, s->dp4, s->cfg.solverIterations == 0 ? 1 : 0, s->ka0, s->va0, s->kb0, s->vb0);
        mark("k_import");
        if (learn_mode(s)) {  // the previous step's lambda sums, in the records' order
            cudaError_t ce = cudaMemcpyAsync(s->lacc, s->lacc_ref, sizeof(float) * s->n,
                                             cudaMemcpyDeviceToDevice, st);
            if (ce != cudaSuccess) return cuda_status(ce);
        }
    }
    if (!import) {  // the state is already on the device: only the sort keys
        akua::k_keys<<<grid_for(s->n, akua::kElemBlock), akua::kElemBlock, 0, st>>>(
            s->d_params, s->x4, s->v4, s->rref, s->ka0, s->va0, s->kb0, s->vb0);
        mark("k_keys");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    if ((s->options & AKUA_PBF_OPT_NO_GRAPH) || prof) {
        enqueue_body(s, st, aos, stride, prof);
    } else {
        const int rc = ensure_graph(s, aos, stride);
        if (rc != AKUA_OK) return rc;
        e = cudaGraphLaunch(s->exec, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
    if (s->cap_feat) {  // one-shot training capture
        e = cudaMemcpyAsync(s->cap_feat, s->feat, sizeof(float) * 8 * s->n,
                            cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->cap_target, s->lacc, sizeof(float) * s->n,
                                cudaMemcpyDeviceToDevice, st);
        s->cap_feat = nullptr;
        s->cap_target = nullptr;
        if (e != cudaSuccess) return cuda_status(e);
    }
    s->state_valid = true;
    s->stepped = true;
    ++s->steps;
    return AKUA_OK;
}

}  // namespace

extern "C" {

void akua_pbf_default_config(akua_pbf_config* c, akua_lambda_corr_params* k) {
    if (c) {
        c->restDensity = 7600.0f;
        c->particle_spacing = 0.05f;
        c->smoothRadius = 0.1f;
        c->spatialHashCellSize = 0.1f;
        c->relaxation = 600.0f;
        c->vorticityEpsilon = 0.00001f;
        c->viscosity = 0.01f;
        c->maxNeighbours = 128;
        c->solverIterations = 4;
        c->gravity[0] = 0.0f;
        c->gravity[1] = -9.8f;
        c->gravity[2] = 0.0f;
    }
    if (k) {
        k->enabled = 1;
        k->k = 0.0001f;
        k->n = 4.0f;
        k->delta_q = 0.03f;
    }
}

}  // extern "C"

namespace {

// A solver for one scene (scenes == nullptr) or for a batch of independent scenes laid out one
// after another in the particle array.
int create_solver(int32_t n, const akua_pbf_config* cfg, const akua_lambda_corr_params* corr,
                  const akua_scene_desc* scenes, int32_t num_scenes, akua_pbf** out) {
    if (!out) return AKUA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!cfg || !corr || n <= 0) return AKUA_ERR_INVALID_ARGUMENT;
    if (cfg->maxNeighbours <= 0 || cfg->solverIterations < 0) return AKUA_ERR_INVALID_ARGUMENT;
    if (!(cfg->smoothRadius > 0.0f) || !(cfg->spatialHashCellSize > 0.0f) ||
        !(cfg->restDensity > 0.0f) || !std::isfinite(cfg->smoothRadius))
        return AKUA_ERR_INVALID_ARGUMENT;
    // PBFSolver.cpp:15: _tableSize = maxNeighbours * numParticles, an int (per scene); a batch's
    // tables sit one after another in one key space of 32 bits.
    if ((int64_t)cfg->maxNeighbours * (int64_t)n > (int64_t)(scenes ? UINT32_MAX : INT_MAX))
        return AKUA_ERR_TOO_LARGE;
    akua_pbf* s = new (std::nothrow) akua_pbf();
    if (!s) return AKUA_ERR_OUT_OF_MEMORY;
    s->n = n;
    s->cfg = *cfg;
    s->corr = *corr;
    s->table_size = (uint32_t)((int64_t)cfg->maxNeighbours * n);
    s->table_alloc = s->table_size;
    cudaGetDevice(&s->device);
    std::vector<uint16_t> sid;
    if (scenes) {
        s->scenes.assign(scenes, scenes + num_scenes);
        uint32_t first = 0;
        sid.resize((size_t)n);
        for (int k = 0; k < num_scenes; ++k) {
            s->scene_first.push_back(first);
            for (int32_t q = 0; q < scenes[k].numParticles; ++q) sid[first + q] = (uint16_t)k;
            first += (uint32_t)scenes[k].numParticles;
        }
        while ((1 << s->scene_bits) < num_scenes) ++s->scene_bits;
    }
    const size_t N = (size_t)n;
    const size_t cap = (size_t)cfg->maxNeighbours;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    chk(dalloc(s, &s->d_params, scenes ? (size_t)num_scenes : 1));
    if (scenes) {
        chk(dalloc(s, &s->scene_of, N));
        if (e == cudaSuccess)
            e = cudaMemcpy(s->scene_of, sid.data(), sizeof(uint16_t) * N, cudaMemcpyHostToDevice);
    }
    chk(dalloc(s, &s->x4, N)); chk(dalloc(s, &s->v4, N)); chk(dalloc(s, &s->col4, N));
    chk(dalloc(s, &s->size, N)); chk(dalloc(s, &s->rref, N));
    chk(dalloc(s, &s->rho, N)); chk(dalloc(s, &s->lam, N)); chk(dalloc(s, &s->dp4, N));
    chk(dalloc(s, &s->x4g, N)); chk(dalloc(s, &s->col4g, N));
    chk(dalloc(s, &s->ps0, N)); chk(dalloc(s, &s->ps1, N));
    chk(dalloc(s, &s->vstar4, N)); chk(dalloc(s, &s->om4, N)); chk(dalloc(s, &s->xv8, 2 * N));
    chk(dalloc(s, &s->dpg, N)); chk(dalloc(s, &s->xref, N));
    chk(dalloc(s, &s->sizeg, N)); chk(dalloc(s, &s->rhog, N)); chk(dalloc(s, &s->lamg, N));
    chk(dalloc(s, &s->rrefg, N)); chk(dalloc(s, &s->rank_of_import, N)); chk(dalloc(s, &s->r2i, N));
    chk(dalloc(s, &s->order, N));
    chk(dalloc(s, &s->ka0, N)); chk(dalloc(s, &s->va0, N));
    chk(dalloc(s, &s->ka1, N)); chk(dalloc(s, &s->va1, N));
    chk(dalloc(s, &s->kb0, N)); chk(dalloc(s, &s->vb0, N));
    chk(dalloc(s, &s->kb1, N)); chk(dalloc(s, &s->vb1, N));
    chk(dalloc(s, &s->sort_scratch, akua::radix::scratch_words(n)));
    chk(dalloc(s, &s->sort_scratch_b, akua::radix::scratch_words(n)));
    chk(dalloc(s, &s->table, (size_t)s->table_alloc));
    chk(dalloc(s, &s->nbr, N * 4 * ((cap + 3) / 4)));  // uint4 tiles of 4 entries
    chk(dalloc(s, &s->cnt, N));
    chk(dalloc(s, &s->flags, 1));
    chk(dalloc(s, &s->psl, N));
    chk(dalloc(s, &s->shapes, AKUA_SDF_MAX_SHAPES));
    chk(dalloc(s, &s->mass_bits, 2));
    if (e == cudaSuccess) e = cudaMemset(s->table, 0, sizeof(uint2) * (size_t)s->table_alloc);
    if (e == cudaSuccess) e = cudaMemset(s->flags, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(s->dp4, 0, sizeof(float4) * N);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
    // every tile shape of the walk fits the default 48 KB of dynamic shared memory
    static_assert(akua::search_smem(256, 32) <= 48 * 1024 && akua::search_smem(128, 48) <= 48 * 1024,
                  "walk staging exceeds 48 KB");
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        free_all(s);
        delete s;
        cudaGetLastError();
        return cuda_status(e);
    }
    update_plans(s, 1);
    *out = s;
    return AKUA_OK;
}

}  // namespace

extern "C" {

int akua_pbf_create(int32_t n, const akua_pbf_config* cfg, const akua_lambda_corr_params* corr,
                    akua_pbf** out) {
    return create_solver(n, cfg, corr, nullptr, 0, out);
}

int akua_pbf_create_batch(int32_t num_scenes, const akua_scene_desc* scenes,
                          const akua_pbf_config* cfg, const akua_lambda_corr_params* corr,
                          akua_pbf** out) {
    if (out) *out = nullptr;
    if (!scenes || num_scenes <= 0 || num_scenes > 65535) return AKUA_ERR_INVALID_ARGUMENT;
    int64_t total = 0;
    for (int k = 0; k < num_scenes; ++k) {
        const akua_scene_desc& d = scenes[k];
        if (d.numParticles <= 0 || !finite3(d.gravity) || !finite3(d.boxMin) || !finite3(d.boxMax))
            return AKUA_ERR_INVALID_ARGUMENT;
        if (cfg && (int64_t)cfg->maxNeighbours * d.numParticles > (int64_t)INT_MAX)
            return AKUA_ERR_TOO_LARGE;
        total += d.numParticles;
    }
    if (total > (int64_t)INT_MAX) return AKUA_ERR_TOO_LARGE;
    return create_solver((int32_t)total, cfg, corr, scenes, num_scenes, out);
}

int akua_pbf_step_batch(akua_pbf* s, float dt) {
    if (!s || s->scenes.empty()) return AKUA_ERR_INVALID_ARGUMENT;
    if (!s->attached) return AKUA_ERR_NOT_ATTACHED;
    DeviceGuard g(s->device);
    return do_step(s, s->attached, s->stride, false, dt, nullptr, nullptr);
}

int akua_pbf_set_scene(akua_pbf* s, int32_t scene, const akua_scene_desc* desc) {
    if (!s || !desc || scene < 0 || scene >= (int32_t)s->scenes.size()) return AKUA_ERR_INVALID_ARGUMENT;
    if (desc->numParticles != s->scenes[scene].numParticles || !finite3(desc->gravity) ||
        !finite3(desc->boxMin) || !finite3(desc->boxMax))
        return AKUA_ERR_INVALID_ARGUMENT;
    s->scenes[scene] = *desc;
    return AKUA_OK;
}

int akua_pbf_destroy(akua_pbf* s) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    int rc = cuda_status(cudaStreamSynchronize(s->stream));
    free_all(s);
    delete s;
    return rc;
}

int akua_pbf_attach_particles(akua_pbf* s, void* dev, size_t stride) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    if (dev && (stride < sizeof(akua_particle) || stride % 4 != 0 ||
                (reinterpret_cast<uintptr_t>(dev) & 3u) != 0))
        return AKUA_ERR_INVALID_ARGUMENT;
    s->attached = static_cast<char*>(dev);
    s->stride = dev ? stride : 0;
    s->state_valid = false;
    return AKUA_OK;
}

int akua_pbf_step(akua_pbf* s, float dt, const float bmin[3], const float bmax[3]) {
    if (!s || !s->scenes.empty()) return AKUA_ERR_INVALID_ARGUMENT;  // batches: akua_pbf_step_batch
    if (!s->attached) return AKUA_ERR_NOT_ATTACHED;
    DeviceGuard g(s->device);
    return do_step(s, s->attached, s->stride, false, dt, bmin, bmax);
}

int akua_pbf_step_host(akua_pbf* s, void* host, size_t stride, float dt, const float bmin[3],
                       const float bmax[3]) {
    if (!s || !host || stride < sizeof(akua_particle) || stride % 4 != 0 || !s->scenes.empty())
        return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    // Pinned records: the import and export kernels read and write them in place over the host
    // link, with no staging copies.  Other host memory goes through a device staging buffer.
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, host) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
        attr.devicePointer) {
        const int rc = do_step(s, static_cast<const char*>(attr.devicePointer), stride, true, dt,
                               bmin, bmax);
        if (rc != AKUA_OK) return rc;
        return cuda_status(cudaStreamSynchronize(s->stream));
    }
    cudaGetLastError();
    const size_t bytes = (size_t)s->n * stride;
    if (s->staging_bytes < bytes) {
        if (s->staging) {
            cudaStreamSynchronize(s->stream);
            cudaFree(s->staging);
            s->device_bytes -= s->staging_bytes;
            s->staging = nullptr;
            s->staging_bytes = 0;
        }
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s->staging), bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            s->staging = nullptr;
            return cuda_status(e);
        }
        s->staging_bytes = bytes;
        s->device_bytes += bytes;
    }
    cudaError_t e = cudaMemcpyAsync(s->staging, host, bytes, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) return cuda_status(e);
    int rc = do_step(s, s->staging, stride, true, dt, bmin, bmax);
    if (rc != AKUA_OK) return rc;
    e = cudaMemcpyAsync(host, s->staging, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e != cudaSuccess) return cuda_status(e);
    return cuda_status(cudaStreamSynchronize(s->stream));
}

int akua_pbf_set_gravity(akua_pbf* s, const float g[3]) {
    if (!s || !finite3(g) || !s->scenes.empty()) return AKUA_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; ++a) s->cfg.gravity[a] = g[a];
    return AKUA_OK;
}

int akua_pbf_set_boundary_damping(akua_pbf* s, float restitution, float friction) {
    if (!s || !std::isfinite(restitution) || !std::isfinite(friction))
        return AKUA_ERR_INVALID_ARGUMENT;
    s->restitution = restitution;
    s->friction = friction;
    return AKUA_OK;
}

int akua_pbf_set_solver_iterations(akua_pbf* s, int32_t iterations) {
    if (!s || iterations < 0 || iterations > 1000) return AKUA_ERR_INVALID_ARGUMENT;
    if ((s->warm || s->cap_feat || s->track) && iterations < 1) return AKUA_ERR_INVALID_ARGUMENT;
    s->cfg.solverIterations = iterations;
    invalidate_graph(s);
    return AKUA_OK;
}

int akua_pbf_set_table_size(akua_pbf* s, int32_t table_size) {
    if (!s || table_size <= 0 || !s->scenes.empty()) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    if ((uint32_t)table_size > s->table_alloc) {
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return cuda_status(e);
        uint2* t = nullptr;
        e = cudaMalloc(reinterpret_cast<void**>(&t), sizeof(uint2) * (size_t)table_size);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_status(e);
        }
        cudaFree(s->table);
        s->device_bytes -= sizeof(uint2) * (size_t)s->table_alloc;
        s->device_bytes += sizeof(uint2) * (size_t)table_size;
        s->table = t;
        s->table_alloc = (uint32_t)table_size;
    }
    // A smaller table reuses the allocation, emptied.
    cudaError_t e = cudaMemsetAsync(s->table, 0, sizeof(uint2) * (size_t)s->table_alloc, s->stream);
    if (e != cudaSuccess) return cuda_status(e);
    s->table_size = (uint32_t)table_size;
    update_plans(s, s->sp_bits);
    invalidate_graph(s);
    return AKUA_OK;
}

int akua_pbf_set_stream(akua_pbf* s, void* stream) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    s->stream = static_cast<cudaStream_t>(stream);
    return AKUA_OK;
}

int akua_pbf_set_options(akua_pbf* s, uint32_t options) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    const uint32_t known = AKUA_PBF_OPT_EXACT_MATH | AKUA_PBF_OPT_RESIDENT | AKUA_PBF_OPT_NO_GRAPH;
    if (options & ~known) return AKUA_ERR_INVALID_ARGUMENT;
    s->options = options;
    return AKUA_OK;
}

int akua_pbf_synchronize(akua_pbf* s) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    return cuda_status(cudaStreamSynchronize(s->stream));
}

int akua_pbf_get_stats(akua_pbf* s, akua_pbf_stats* st) {
    if (!s || !st) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t flags = 0;
    e = cudaMemcpy(&flags, s->flags, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    st->numParticles = s->n;
    st->tableSize = (int32_t)s->table_size;
    st->maxNeighbours = s->cfg.maxNeighbours;
    st->solverIterations = s->cfg.solverIterations;
    st->steps = s->steps;
    st->deviceFlags = flags;
    st->graphCaptures = s->graph_captures;
    st->deviceBytes = s->device_bytes;
    return AKUA_OK;
}

int akua_pbf_read_debug(akua_pbf* s, int32_t what, void* dst, size_t bytes) {
    if (!s || !dst) return AKUA_ERR_INVALID_ARGUMENT;
    if (!s->stepped) return AKUA_ERR_INVALID_ARGUMENT;  // nothing computed yet
    DeviceGuard g(s->device);
    const size_t N = (size_t)s->n;
    const size_t cap = (size_t)s->cfg.maxNeighbours;
    size_t need = 0;
    switch (what) {
        case AKUA_DEBUG_HASHES:
        case AKUA_DEBUG_ORDER:
        case AKUA_DEBUG_NEIGHBOUR_COUNTS:
        case AKUA_DEBUG_LAMBDA_SUMS: need = N * 4; break;
        case AKUA_DEBUG_NEIGHBOURS: need = N * cap * 4; break;
        case AKUA_DEBUG_PARTICLES: need = N * sizeof(akua_particle); break;
        default: return AKUA_ERR_INVALID_ARGUMENT;
    }
    if (bytes != need) return AKUA_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_status(e);
    if (what == AKUA_DEBUG_HASHES) return cuda_status(cudaMemcpy(dst, s->kr, need, cudaMemcpyDeviceToHost));
    if (what == AKUA_DEBUG_LAMBDA_SUMS) {
        if (!s->lacc_ref) {
            std::memset(dst, 0, need);
            return AKUA_OK;
        }
        return cuda_status(cudaMemcpy(dst, s->lacc_ref, need, cudaMemcpyDeviceToHost));
    }
    if (what == AKUA_DEBUG_ORDER) return cuda_status(cudaMemcpy(dst, s->order, need, cudaMemcpyDeviceToHost));
    if (what == AKUA_DEBUG_PARTICLES) {
        char* tmp = nullptr;
        e = cudaMalloc(reinterpret_cast<void**>(&tmp), need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cuda_status(e);
        }
        akua::k_export<<<grid_for(s->n, akua::kIoBlock), akua::kIoBlock, 0, s->stream>>>(
            s->d_params, tmp, sizeof(akua_particle), s->n, s->r2i, s->kr, s->x4, s->v4, s->vstar4, s->dp4,
            s->om4, s->rho, s->lam, s->col4, s->size, nullptr, nullptr);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, tmp, need, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        cudaFree(tmp);
        return cuda_status(e);
    }
    // Neighbour data: convert internal indices to reference ranks (the reference's indexing).
    std::vector<uint32_t> r2i(N), rank(N), cnt(N);
    e = cudaMemcpy(r2i.data(), s->r2i, N * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(rank.data(), s->rref, N * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cnt.data(), s->cnt, N * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t* out = static_cast<uint32_t*>(dst);
    if (what == AKUA_DEBUG_NEIGHBOUR_COUNTS) {
        for (size_t r = 0; r < N; ++r) out[r] = cnt[r2i[r]];
        return AKUA_OK;
    }
    const size_t words = N * 4 * ((cap + 3) / 4);
    std::vector<uint32_t> nbr(words);
    e = cudaMemcpy(nbr.data(), s->nbr, words * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e);
    std::memset(out, 0, need);
    for (size_t r = 0; r < N; ++r) {
        const uint32_t i = r2i[r];
        for (uint32_t k = 0; k < cnt[i] && k < cap; ++k)
            out[r * cap + k] = rank[nbr[4 * ((size_t)(k >> 2) * N + i) + (k & 3)]];
    }
    return AKUA_OK;
}

int akua_pbf_kernels_per_step(akua_pbf* s) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    if (s->body_launches == 0) return AKUA_ERR_INVALID_ARGUMENT;  // no step issued yet
    // parameter upload (one launch per chunk of scenes) + import or the sort keys + the body
    const int uploads =
        s->scenes.empty() ? 1 : (int)((s->scenes.size() + akua::kParamChunk - 1) / akua::kParamChunk);
    return uploads + 1 + s->body_launches;
}

int akua_pbf_profile_begin(akua_pbf* s, int32_t max_steps) {
    if (!s || max_steps <= 0 || max_steps > 100000) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    for (cudaEvent_t ev : s->prof_events) cudaEventDestroy(ev);
    s->prof_events.clear();
    const size_t per_step = 16 + 3 * (size_t)(akua::radix::MAX_PASSES * 2) +
                            2 * (size_t)s->cfg.solverIterations;
    const size_t total = per_step * (size_t)max_steps;
    s->prof_events.resize(total, nullptr);
    s->prof_names.assign(total, nullptr);
    for (size_t i = 0; i < total; ++i) {
        cudaError_t e = cudaEventCreate(&s->prof_events[i]);
        if (e != cudaSuccess) {
            s->prof_events.resize(i);
            return cuda_status(e);
        }
    }
    s->prof_next = 0;
    s->prof_steps_left = max_steps;
    s->prof_active = true;
    return AKUA_OK;
}

int akua_pbf_profile_end(akua_pbf* s, akua_kernel_time* out, int32_t capacity, int32_t* count) {
    if (!s || !count || (capacity > 0 && !out)) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    std::map<std::string, std::pair<int, double>> acc;
    std::vector<std::string> order;
    for (size_t i = 1; e == cudaSuccess && i < s->prof_next; ++i) {
        const char* name = s->prof_names[i];
        if (!name) continue;  // start of a step: nothing ran since the previous event
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, s->prof_events[i - 1], s->prof_events[i]);
        if (e != cudaSuccess) break;
        auto it = acc.find(name);
        if (it == acc.end()) {
            order.push_back(name);
            acc[name] = {1, (double)ms};
        } else {
            it->second.first += 1;
            it->second.second += ms;
        }
    }
    for (cudaEvent_t ev : s->prof_events) cudaEventDestroy(ev);
    s->prof_events.clear();
    s->prof_names.clear();
    s->prof_next = 0;
    s->prof_active = false;
    s->prof_steps_left = 0;
    if (e != cudaSuccess) return cuda_status(e);
    int32_t k = 0;
    for (const std::string& name : order) {
        if (k < capacity) {
            std::snprintf(out[k].name, sizeof(out[k].name), "%s", name.c_str());
            out[k].launches = acc[name].first;
            out[k].total_ms = acc[name].second;
        }
        ++k;
    }
    *count = k;
    return AKUA_OK;
}

int akua_pbf_set_warm_start(akua_pbf* s, akua_mlp* net) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    if (net && (net->device != s->device || s->cfg.solverIterations < 1))
        return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    if (net) {
        const cudaError_t e = ensure_learn_buffers(s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    s->warm = net;
    return AKUA_OK;
}

int akua_pbf_capture_training(akua_pbf* s, float* features, float* targets) {
    if (!s || (!features) != (!targets)) return AKUA_ERR_INVALID_ARGUMENT;
    if (features && s->cfg.solverIterations < 1) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    if (features) {
        const cudaError_t e = ensure_learn_buffers(s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    s->cap_feat = features;
    s->cap_target = targets;
    if (features) s->track = true;
    return AKUA_OK;
}

int akua_pbf_set_lambda_tracking(akua_pbf* s, int32_t enabled) {
    if (!s) return AKUA_ERR_INVALID_ARGUMENT;
    if (enabled && s->cfg.solverIterations < 1) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    if (enabled) {
        const cudaError_t e = ensure_learn_buffers(s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    s->track = enabled != 0;
    return AKUA_OK;
}

int akua_pbf_set_pair_blocks(akua_pbf* s, const int32_t blocks[AKUA_PBF_PAIR_KERNELS]) {
    if (!s || !blocks) return AKUA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k)
        if (blocks[k] != 64 && blocks[k] != 128 && blocks[k] != 256)
            return AKUA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) s->pair_block[k] = blocks[k];
    invalidate_graph(s);
    return AKUA_OK;
}

int akua_pbf_get_pair_blocks(akua_pbf* s, int32_t blocks[AKUA_PBF_PAIR_KERNELS]) {
    if (!s || !blocks) return AKUA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) blocks[k] = s->pair_block[k];
    return AKUA_OK;
}

int akua_pbf_set_search_shape(akua_pbf* s, int32_t block, int32_t staged) {
    if (!s || (block != 64 && block != 128 && block != 256) ||
        (staged != 16 && staged != 32 && staged != 48) || (staged == 48 && block == 256))
        return AKUA_ERR_INVALID_ARGUMENT;
    s->search_block = block;
    s->search_stage = staged;
    invalidate_graph(s);
    return AKUA_OK;
}

int akua_pbf_get_search_shape(akua_pbf* s, int32_t* block, int32_t* staged) {
    if (!s || !block || !staged) return AKUA_ERR_INVALID_ARGUMENT;
    *block = s->search_block;
    *staged = s->search_stage;
    return AKUA_OK;
}

int akua_pbf_autotune(akua_pbf* s, float dt, const float bmin[3], const float bmax[3],
                      int32_t steps, int32_t* blocks_out) {
    if (!s || steps <= 0 || steps > 100) return AKUA_ERR_INVALID_ARGUMENT;
    if (!s->attached) return AKUA_ERR_NOT_ATTACHED;
    DeviceGuard g(s->device);
    static const char* const names[AKUA_PBF_PAIR_KERNELS] = {
        "k_density_lambda", "k_delta_correct", "k_delta_final", "k_vorticity", "k_confine",
        "k_xsph"};
    const int cands[3] = {64, 128, 256};
    const size_t bytes = (size_t)s->n * s->stride;
    char* const user = s->attached;
    const int64_t steps0 = s->steps;
    float* const cap_f = s->cap_feat;
    float* const cap_t = s->cap_target;
    s->cap_feat = s->cap_target = nullptr;
    char* tmp = nullptr;
    float* sums = nullptr;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&tmp), bytes);
    if (e == cudaSuccess && s->lacc_ref)
        e = cudaMalloc(reinterpret_cast<void**>(&sums), sizeof(float) * (size_t)s->n);
    if (e == cudaSuccess && sums)
        e = cudaMemcpy(sums, s->lacc_ref, sizeof(float) * (size_t)s->n, cudaMemcpyDeviceToDevice);
    int rc = cuda_status(e);
    double best[AKUA_PBF_PAIR_KERNELS];
    int choice[AKUA_PBF_PAIR_KERNELS];
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) {
        best[k] = 1e30;
        choice[k] = s->pair_block[k];
    }
    std::vector<akua_kernel_time> times(64);
    int32_t count = 0;
    // one timed trial of the current launch shapes from a copy of the user's records
    auto trial = [&]() {
        invalidate_graph(s);
        // every candidate starts from the same records (and lambda sums)
        e = cudaMemcpy(tmp, user, bytes, cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess && sums)
            e = cudaMemcpy(s->lacc_ref, sums, sizeof(float) * (size_t)s->n,
                           cudaMemcpyDeviceToDevice);
        rc = cuda_status(e);
        if (rc == AKUA_OK) rc = do_step(s, tmp, s->stride, true, dt, bmin, bmax);
        if (rc == AKUA_OK) rc = akua_pbf_profile_begin(s, steps);
        for (int k = 0; k < steps && rc == AKUA_OK; ++k)
            rc = do_step(s, tmp, s->stride, false, dt, bmin, bmax);
        count = 0;
        const int rc_end = akua_pbf_profile_end(s, times.data(), (int32_t)times.size(), &count);
        if (rc == AKUA_OK) rc = rc_end;
    };
    auto per_launch = [&](const char* name) {
        for (int t = 0; t < count; ++t)
            if (std::strcmp(times[t].name, name) == 0 && times[t].launches > 0)
                return times[t].total_ms / times[t].launches;
        return 1e30;
    };
    for (int c = 0; c < 3 && rc == AKUA_OK; ++c) {
        for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) s->pair_block[k] = cands[c];
        trial();
        for (int k = 0; k < AKUA_PBF_PAIR_KERNELS && rc == AKUA_OK; ++k) {
            const double per = per_launch(names[k]);
            if (per < best[k]) {
                best[k] = per;
                choice[k] = cands[c];
            }
        }
    }
    // the walk's tile shape, with the pair kernels at their chosen sizes
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) s->pair_block[k] = choice[k];
    const int shapes[8][2] = {{128, 32}, {64, 32}, {256, 32}, {128, 16}, {64, 16}, {256, 16},
                              {64, 48}, {128, 48}};
    int shape_choice[2] = {s->search_block, s->search_stage};
    double shape_best = 1e30;
    for (int c = 0; c < 8 && rc == AKUA_OK; ++c) {
        s->search_block = shapes[c][0];
        s->search_stage = shapes[c][1];
        trial();
        const double per = per_launch("k_search");
        if (rc == AKUA_OK && per < shape_best) {
            shape_best = per;
            shape_choice[0] = shapes[c][0];
            shape_choice[1] = shapes[c][1];
        }
    }
    s->search_block = shape_choice[0];
    s->search_stage = shape_choice[1];
    for (int k = 0; k < AKUA_PBF_PAIR_KERNELS; ++k) {
        s->pair_block[k] = choice[k];
        if (blocks_out) blocks_out[k] = choice[k];
    }
    invalidate_graph(s);
    if (sums) {
        cudaMemcpy(s->lacc_ref, sums, sizeof(float) * (size_t)s->n, cudaMemcpyDeviceToDevice);
        cudaFree(sums);
    }
    if (tmp) cudaFree(tmp);
    s->attached = user;
    s->steps = steps0;
    s->state_valid = false;  // the next step imports the user's records again
    s->cap_feat = cap_f;
    s->cap_target = cap_t;
    return rc;
}

int akua_pbf_set_sdf_shapes(akua_pbf* s, const akua_sdf_shape* shapes, int32_t count,
                            float minDist, float stiffness) {
    if (!s || count < 0 || count > AKUA_SDF_MAX_SHAPES || (count > 0 && !shapes) ||
        !std::isfinite(minDist) || !std::isfinite(stiffness))
        return AKUA_ERR_INVALID_ARGUMENT;
    static_assert(sizeof(akua_sdf_shape) == sizeof(akua::SdfShape), "shape layout");
    for (int k = 0; k < count; ++k) {
        const akua_sdf_shape& d = shapes[k];
        if (d.type < AKUA_SDF_SPHERE || d.type > AKUA_SDF_PLANE || !finite3(d.a) || !finite3(d.b) ||
            !std::isfinite(d.radius))
            return AKUA_ERR_INVALID_ARGUMENT;
    }
    DeviceGuard g(s->device);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && count > 0)
        e = cudaMemcpy(s->shapes, shapes, sizeof(akua_sdf_shape) * (size_t)count,
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e);
    s->num_shapes = count;
    s->sdf_min_dist = minDist;
    s->sdf_stiffness = stiffness;
    return AKUA_OK;
}

int akua_pbf_set_lambda_sums(akua_pbf* s, const float* host, int64_t count) {
    if (!s || !host || count != (int64_t)s->n) return AKUA_ERR_INVALID_ARGUMENT;
    DeviceGuard g(s->device);
    cudaError_t e = ensure_learn_buffers(s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->lacc_ref, host, sizeof(float) * (size_t)count, cudaMemcpyHostToDevice);
    s->state_valid = false;  // the next step re-imports records and sums together
    return cuda_status(e);
}

int akua_pbf_density_error(akua_pbf* s, float* max_error, float* mean_abs_error) {
    if (!s || !max_error || !mean_abs_error) return AKUA_ERR_INVALID_ARGUMENT;
    if (!s->stepped) return AKUA_ERR_NOT_ATTACHED;
    DeviceGuard g(s->device);
    cudaError_t e = ensure_learn_buffers(s);
    cudaStream_t st = s->stream;
    if (e == cudaSuccess) e = cudaMemsetAsync(s->err_max, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->err_sum, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_status(e);
    akua::k_density_error<<<grid_for(s->n, akua::kPairBlock), akua::kPairBlock, 0, st>>>(
        s->d_params, s->x4, reinterpret_cast<const uint4*>(s->nbr), s->cnt, s->err_max,
        s->err_sum);
    uint32_t bits = 0;
    double sum = 0.0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, s->err_max, sizeof(bits), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&sum, s->err_sum, sizeof(sum), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    float m;
    std::memcpy(&m, &bits, sizeof(m));
    *max_error = m;
    *mean_abs_error = (float)(sum / (double)s->n);
    return AKUA_OK;
}

const char* akua_pbf_status_string(int status) {
    switch (status) {
        case AKUA_OK: return "ok";
        case AKUA_ERR_INVALID_ARGUMENT: return "invalid argument";
        case AKUA_ERR_CUDA: return "CUDA error";
        case AKUA_ERR_OUT_OF_MEMORY: return "out of device memory";
        case AKUA_ERR_NOT_ATTACHED: return "no particle buffer attached";
        case AKUA_ERR_DEVICE_CHECK: return "device-side check failed";
        case AKUA_ERR_TOO_LARGE: return "size exceeds the entry point's limit";
        case AKUA_ERR_CORRUPT: return "state file failed its checksum";
        default: return "unknown status";
    }
}

int akua_pbf_abi_version(void) { return AKUA_PBF_ABI_VERSION; }

}  // extern "C"
