// Bounded mbarrier waits of the tensor-core kernels (akuaengine_gb300/csrc/tc05.cuh): a wait on a
// phase that never completes must return false after its try limit, a wait on a completed phase
// must return true, and the context must stay usable afterwards.  Prints one JSON line.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "tc05.cuh"

namespace {

__global__ void k_wait(int arrive, uint32_t max_tries, uint32_t* result, long long* cycles) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) akua::tc::mbar_init(&bar, 1);
    __syncthreads();
    if (arrive && threadIdx.x == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(akua::tc::smem_addr(&bar))
                     : "memory");
    __syncthreads();
    const long long t0 = clock64();
    const bool ok = akua::tc::mbar_wait(&bar, 0, max_tries);  // phase 0
    const long long t1 = clock64();
    if (threadIdx.x == 0) {
        *result = ok ? 1u : 0u;
        *cycles = t1 - t0;
    }
}

__global__ void k_add(int* x) { atomicAdd(x, 1); }

}  // namespace

int main() {
    uint32_t* r = nullptr;
    long long* c = nullptr;
    int* x = nullptr;
    if (cudaMalloc(&r, 2 * sizeof(uint32_t)) != cudaSuccess || cudaMalloc(&c, 2 * sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&x, sizeof(int)) != cudaSuccess) {
        std::printf("{\"error\": \"allocation\"}\n");
        return 1;
    }
    cudaMemset(r, 0xff, 2 * sizeof(uint32_t));
    cudaMemset(x, 0, sizeof(int));
    k_wait<<<1, 32>>>(0, 4096, r, c);      // nothing arrives: must time out
    k_wait<<<1, 32>>>(1, 4096, r + 1, c + 1);  // one arrival completes phase 0
    k_add<<<4, 32>>>(x);                    // the context still runs kernels
    const cudaError_t e = cudaDeviceSynchronize();
    uint32_t hr[2] = {9, 9};
    long long hc[2] = {0, 0};
    int hx = 0;
    cudaMemcpy(hr, r, sizeof(hr), cudaMemcpyDeviceToHost);
    cudaMemcpy(hc, c, sizeof(hc), cudaMemcpyDeviceToHost);
    cudaMemcpy(&hx, x, sizeof(hx), cudaMemcpyDeviceToHost);
    std::printf("{\"sync\": \"%s\", \"timeout_result\": %u, \"arrived_result\": %u, "
                "\"timeout_cycles\": %lld, \"arrived_cycles\": %lld, \"after\": %d}\n",
                cudaGetErrorName(e), hr[0], hr[1], hc[0], hc[1], hx);
    return e == cudaSuccess ? 0 : 1;
}
