// Steps a particle file through the C++ host interface (include/akua/PBFSolver.hpp), the way the
// reference's Application::run drives PBFSolver::step once per frame (Application.cpp:66).
//
//   pbf_cpp_steps <in.bin> <out.bin> <steps> <host|device>
//
// in.bin: seven floats (dt, boxMin[3], boxMax[3]) followed by N packed 108-byte particle records;
// out.bin: the N records after the steps.  Solver parameters are the reference defaults.
#include <akua/PBFSolver.hpp>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: %s in.bin out.bin steps host|device\n", argv[0]);
        return 2;
    }
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    float hdr[7];
    if (std::fread(hdr, sizeof(float), 7, f) != 7) return 2;
    std::vector<akua::Particle> p;
    akua::Particle rec;
    while (std::fread(&rec, sizeof(rec), 1, f) == 1) p.push_back(rec);
    std::fclose(f);
    const int steps = std::atoi(argv[3]);
    const bool device = std::strcmp(argv[4], "device") == 0;
    const akua::Vec3 lo{hdr[1], hdr[2], hdr[3]}, hi{hdr[4], hdr[5], hdr[6]};
    try {
        akua::PBFSolver solver((int)p.size(), akua::PBFConfig{}, akua::LambdaCorrParams{});
        if (device) {
            void* d = nullptr;
            const size_t bytes = p.size() * sizeof(akua::Particle);
            if (cudaMalloc(&d, bytes) != cudaSuccess) return 3;
            cudaMemcpy(d, p.data(), bytes, cudaMemcpyHostToDevice);
            for (int s = 0; s < steps; ++s) solver.step(akua::DeviceParticles{d}, hdr[0], lo, hi);
            solver.synchronize();
            cudaMemcpy(p.data(), d, bytes, cudaMemcpyDeviceToHost);
            cudaFree(d);
        } else {
            for (int s = 0; s < steps; ++s) solver.stepHost(p.data(), hdr[0], lo, hi);
        }
        std::printf("steps %lld particles %d\n", (long long)solver.stats().steps,
                    solver.numParticles());
    } catch (const akua::Error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 4;
    }
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(p.data(), sizeof(akua::Particle), p.size(), f);
    std::fclose(f);
    return 0;
}
