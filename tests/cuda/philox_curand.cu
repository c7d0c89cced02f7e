// Test-only: evaluates curand's Philox4x32-10 block function (called, not
// copied) for a list of counters/keys, to pin the oracle's restatement.
#include <cuda_runtime.h>
#include <curand_kernel.h>

__global__ void k_curand_philox(const uint4* ctr, const uint2* key, uint4* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = curand_Philox4x32_10(ctr[i], key[i]);
}

extern "C" int curand_philox_blocks(const unsigned* ctr, const unsigned* key, unsigned* out, int n) {
    uint4 *dc = nullptr, *dout = nullptr;
    uint2* dk = nullptr;
    if (cudaMalloc(&dc, sizeof(uint4) * n) != cudaSuccess) return -1;
    if (cudaMalloc(&dk, sizeof(uint2) * n) != cudaSuccess) return -1;
    if (cudaMalloc(&dout, sizeof(uint4) * n) != cudaSuccess) return -1;
    cudaMemcpy(dc, ctr, sizeof(uint4) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dk, key, sizeof(uint2) * n, cudaMemcpyHostToDevice);
    k_curand_philox<<<(n + 127) / 128, 128>>>(dc, dk, dout, n);
    cudaError_t e = cudaMemcpy(out, dout, sizeof(uint4) * n, cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dk);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : -2;
}
