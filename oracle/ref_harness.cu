// TEST INFRASTRUCTURE ONLY — never linked into the product.
//
// Runs the reference's own PBF kernels (device code compiled unchanged from the reference's
// src/CUDA/*.cu into cubins by oracle/ref_gpu.py) on a device array of particle records,
// re-sequencing PBFSolver::step (src/Simulation/PBFSolver.cpp:22-78) without the OpenGL map/unmap:
//   predict -> hashes (cell = smoothRadius) -> thrust::sort by hash -> bucket table ->
//   neighbours -> iterations x (densities, lambdas, deltas, correct) -> update ->
//   damping(0, 0.95) -> vorticity -> confinement -> XSPH,
// each launch with the wrappers' 256-thread blocks, followed by cudaDeviceSynchronize.
// --mode faithful additionally reproduces the wrappers' memory traffic: the neighbour arrays live in
// host vectors and are copied to the device in three wrappers and back in one, and the
// tableSize-entry hash table is allocated, filled and freed every step
// (NeighbourSearchCUDA.cu:151-158, 182-183; ConstraintSolverCUDA.cu:195-196;
// IntegrationCUDA.cu:269-270).
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

struct Particle {  // Particle.h:8-31
    float position[3], velocity[3], new_position[3], new_velocity[3], position_delta[3],
        vorticity[3];
    float mass, density, lambda;
    uint32_t hash;
    float color[4];
    float size;
};
static_assert(sizeof(Particle) == 108, "Particle layout");
struct Vec3 {  // glm::vec3 passed by value
    float x, y, z;
};
struct CorrParams {  // LambdaCorrParams (PBFConfig.h:10-15) passed by value
    bool enabled;
    float k, n, delta_q;
};
static_assert(sizeof(CorrParams) == 16, "LambdaCorrParams layout");

struct HashLess {  // the reference's comparator (NeighbourSearchCUDA.cu:168-170)
    __host__ __device__ bool operator()(const Particle& a, const Particle& b) const {
        return a.hash < b.hash;
    }
};

#define CK(x)                                                                              \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
            std::exit(2);                                                                  \
        }                                                                                  \
    } while (0)
#define CU(x)                                                                 \
    do {                                                                      \
        CUresult r_ = (x);                                                    \
        if (r_ != CUDA_SUCCESS) {                                             \
            const char* s_ = nullptr;                                         \
            cuGetErrorString(r_, &s_);                                        \
            std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, s_ ? s_ : "?"); \
            std::exit(3);                                                     \
        }                                                                     \
    } while (0)

static std::map<std::string, CUfunction> g_fn;

static void load_module(const std::string& path) {
    CUmodule mod;
    CU(cuModuleLoad(&mod, path.c_str()));
    unsigned int count = 0;
    CU(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fns(count);
    CU(cuModuleEnumerateFunctions(fns.data(), count, mod));
    const char* wanted[] = {"kernel_predict_position", "kernel_update_position_and_velocity",
                            "kernel_apply_boundary_velocity_damping", "kernel_compute_vorticities",
                            "kernel_apply_vorticity_confinement", "kernel_apply_xsph_viscosity",
                            "kernel_compute_hashes", "kernel_build_hash_table",
                            "kernel_find_neighbours", "kernel_calculate_densities",
                            "kernel_calculate_lambdas", "kernel_calculate_position_delta",
                            "kernel_correct_position"};
    for (CUfunction f : fns) {
        const char* name = nullptr;
        CU(cuFuncGetName(&name, f));
        for (const char* w : wanted)
            if (name && std::strstr(name, w)) g_fn[w] = f;
    }
}

template <class... A>
static void launch(const char* name, int n, A... args) {
    auto it = g_fn.find(name);
    if (it == g_fn.end()) {
        std::fprintf(stderr, "kernel %s not found\n", name);
        std::exit(4);
    }
    void* ptrs[] = {static_cast<void*>(&args)...};
    const int block = 256, grid = (n + block - 1) / block;
    CU(cuLaunchKernel(it->second, grid, 1, 1, block, 1, 1, 0, nullptr, ptrs, nullptr));
    CK(cudaDeviceSynchronize());
}

struct Args {
    std::string cubins, in, out, lists, mode = "resident";
    int n = 0, steps = 1, cap = 128, iters = 4, table = 0, warmup = 0;
    float h = 0.1f, cell = 0.1f, rho0 = 7600.f, relax = 600.f, veps = 1e-5f, visc = 0.01f;
    float k = 1e-4f, nexp = 4.f, dq = 0.03f, dt = 0.0083f;
    Vec3 g{0.f, -9.8f, 0.f}, bmin{0, 0, 0}, bmax{1, 1, 1};
};

static Vec3 parse3(const char* s) {
    Vec3 v{};
    std::sscanf(s, "%f,%f,%f", &v.x, &v.y, &v.z);
    return v;
}

int main(int argc, char** argv) {
    Args a;
    for (int i = 1; i + 1 < argc; i += 2) {
        const std::string k = argv[i];
        const char* v = argv[i + 1];
        if (k == "--cubins") a.cubins = v;
        else if (k == "--in") a.in = v;
        else if (k == "--out") a.out = v;
        else if (k == "--lists") a.lists = v;
        else if (k == "--mode") a.mode = v;
        else if (k == "--n") a.n = std::atoi(v);
        else if (k == "--steps") a.steps = std::atoi(v);
        else if (k == "--warmup") a.warmup = std::atoi(v);
        else if (k == "--cap") a.cap = std::atoi(v);
        else if (k == "--iters") a.iters = std::atoi(v);
        else if (k == "--table") a.table = std::atoi(v);
        else if (k == "--h") a.h = std::strtof(v, nullptr);
        else if (k == "--cell") a.cell = std::strtof(v, nullptr);
        else if (k == "--rho0") a.rho0 = std::strtof(v, nullptr);
        else if (k == "--relax") a.relax = std::strtof(v, nullptr);
        else if (k == "--veps") a.veps = std::strtof(v, nullptr);
        else if (k == "--visc") a.visc = std::strtof(v, nullptr);
        else if (k == "--k") a.k = std::strtof(v, nullptr);
        else if (k == "--nexp") a.nexp = std::strtof(v, nullptr);
        else if (k == "--dq") a.dq = std::strtof(v, nullptr);
        else if (k == "--dt") a.dt = std::strtof(v, nullptr);
        else if (k == "--g") a.g = parse3(v);
        else if (k == "--bmin") a.bmin = parse3(v);
        else if (k == "--bmax") a.bmax = parse3(v);
        else {
            std::fprintf(stderr, "unknown option %s\n", k.c_str());
            return 1;
        }
    }
    const int n = a.n;
    if (n <= 0 || a.in.empty() || a.out.empty() || a.cubins.empty()) return 1;
    if (a.table <= 0) a.table = a.cap * n;  // PBFSolver.cpp:15
    CK(cudaFree(nullptr));
    for (const char* u : {"NeighbourSearchCUDA", "ConstraintSolverCUDA", "IntegrationCUDA"})
        load_module(a.cubins + "/" + u + ".cubin");

    std::vector<Particle> host(n);
    FILE* f = std::fopen(a.in.c_str(), "rb");
    if (!f || std::fread(host.data(), sizeof(Particle), n, f) != (size_t)n) return 5;
    std::fclose(f);
    Particle* d = nullptr;
    CK(cudaMalloc(&d, sizeof(Particle) * n));
    CK(cudaMemcpy(d, host.data(), sizeof(Particle) * n, cudaMemcpyHostToDevice));

    const bool faithful = a.mode == "faithful";
    const size_t lw = (size_t)n * a.cap;
    std::vector<uint32_t> h_nbr(lw, 0u), h_cnt(n, 0u);  // PBFSolver.h:23-24
    uint32_t *nbr = nullptr, *cnt = nullptr, *tbl = nullptr;
    if (!faithful) {
        CK(cudaMalloc(&nbr, lw * 4));
        CK(cudaMalloc(&cnt, (size_t)n * 4));
        CK(cudaMalloc(&tbl, (size_t)a.table * 4));
    }
    const float inv = 1.0f / a.rho0;  // ConstraintSolverCUDA.cu:201
    const CorrParams corr{true, a.k, a.nexp, a.dq};
    const int N = n, cap = a.cap, table = a.table;

    auto to_dev = [&]() {
        CK(cudaMalloc(&nbr, lw * 4));
        CK(cudaMalloc(&cnt, (size_t)n * 4));
        CK(cudaMemcpy(nbr, h_nbr.data(), lw * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(cnt, h_cnt.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    };
    auto free_dev = [&]() {
        CK(cudaFree(nbr));
        CK(cudaFree(cnt));
        nbr = cnt = nullptr;
    };

    auto step = [&]() {
        launch("kernel_predict_position", N, d, N, a.dt, a.g);
        // findParticleNeighboursCUDA
        if (faithful) {
            to_dev();
            CK(cudaMalloc(&tbl, (size_t)table * 4));
        }
        CK(cudaMemset(tbl, 0xff, (size_t)table * 4));
        launch("kernel_compute_hashes", N, d, N, a.h, table);
        thrust::sort(thrust::device, d, d + N, HashLess());
        CK(cudaDeviceSynchronize());
        launch("kernel_build_hash_table", N, d, N, tbl);
        launch("kernel_find_neighbours", N, d, N, nbr, cnt, tbl, a.cell, a.h, table, cap);
        if (faithful) {
            CK(cudaMemcpy(h_nbr.data(), nbr, lw * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(h_cnt.data(), cnt, (size_t)n * 4, cudaMemcpyDeviceToHost));
            CK(cudaFree(tbl));
            tbl = nullptr;
            free_dev();
            to_dev();  // runConstraintSolverCUDA
        }
        for (int it = 0; it < a.iters; ++it) {
            launch("kernel_calculate_densities", N, d, N, nbr, cnt, a.h, cap);
            launch("kernel_calculate_lambdas", N, d, N, nbr, cnt, a.h, cap, inv, a.relax);
            launch("kernel_calculate_position_delta", N, d, N, nbr, cnt, a.h, cap, inv, corr);
            launch("kernel_correct_position", N, d, N, a.bmin, a.bmax);
        }
        if (faithful) free_dev();
        launch("kernel_update_position_and_velocity", N, d, N, a.dt);
        launch("kernel_apply_boundary_velocity_damping", N, d, N, a.bmin, a.bmax, 0.0f, 0.95f);
        if (faithful) to_dev();  // applyVorticityAndViscosityCUDA
        launch("kernel_compute_vorticities", N, d, N, nbr, cnt, a.h, cap);
        launch("kernel_apply_vorticity_confinement", N, d, N, nbr, cnt, cap, a.h, a.dt, a.veps);
        launch("kernel_apply_xsph_viscosity", N, d, N, nbr, cnt, cap, a.h, a.visc);
        if (faithful) free_dev();
    };

    for (int s = 0; s < a.warmup; ++s) step();
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0));
    for (int s = 0; s < a.steps; ++s) {
        // the last step keeps its lists on the device for the dump
        step();
    }
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    std::printf("ms_per_step %.6f\n", ms / (a.steps > 0 ? a.steps : 1));

    CK(cudaMemcpy(host.data(), d, sizeof(Particle) * n, cudaMemcpyDeviceToHost));
    f = std::fopen(a.out.c_str(), "wb");
    if (!f || std::fwrite(host.data(), sizeof(Particle), n, f) != (size_t)n) return 6;
    std::fclose(f);
    if (!a.lists.empty()) {
        if (!faithful) {
            CK(cudaMemcpy(h_nbr.data(), nbr, lw * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(h_cnt.data(), cnt, (size_t)n * 4, cudaMemcpyDeviceToHost));
        }
        FILE* g1 = std::fopen((a.lists + ".nbr").c_str(), "wb");
        FILE* g2 = std::fopen((a.lists + ".cnt").c_str(), "wb");
        if (!g1 || !g2) return 7;
        std::fwrite(h_nbr.data(), 4, lw, g1);
        std::fwrite(h_cnt.data(), 4, n, g2);
        std::fclose(g1);
        std::fclose(g2);
    }
    return 0;
}
