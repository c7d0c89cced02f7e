// isg_common.cuh — shared device/host helpers of libisinggb (sm_103a).
//
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw, SC'11):
// it replaces the per-thread curandState (48 B loaded and stored per update in
// src/cuda/kernels.cu:49-51) with pure arithmetic on a counter, so random
// numbers cost no memory traffic and any site's stream can be replayed.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "isg.h"

#define ISG_FULL_MASK 0xFFFFFFFFu

namespace isg {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

struct U4 {
    uint32_t x, y, z, w;
};

// Ten rounds; the key schedule is folded into the loop so that warp-uniform
// keys stay in uniform registers.
__device__ __forceinline__ U4 philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                       uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(kPhiloxM0, c0);
        const uint32_t lo0 = kPhiloxM0 * c0;
        const uint32_t hi1 = __umulhi(kPhiloxM1, c2);
        const uint32_t lo1 = kPhiloxM1 * c2;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return U4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ uint32_t counter_word3(uint32_t tag, uint32_t colour,
                                                           uint64_t step) {
    return (tag << 24) | (colour << 16) | ((uint32_t)(step >> 32) & 0xFFFFu);
}

__host__ __device__ __forceinline__ uint32_t replica_uid(int L, int r) {
    return ((uint32_t)L << 16) | (uint32_t)r;
}
__host__ __device__ __forceinline__ uint32_t exchange_uid(int L) {
    return ((uint32_t)L << 16) | 0xFFFFu;
}

// 53-bit uniform double in [0,1) from two words.
__device__ __forceinline__ double uniform53(uint32_t w0, uint32_t w1) {
    const uint64_t x = ((uint64_t)w0 << 32) | w1;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// 24-bit uniform float in [0,1) from one word.
__device__ __forceinline__ float uniform24(uint32_t w) {
    return (float)(w >> 8) * (1.0f / 16777216.0f);
}

// n / d for n < 2^31 and a fixed divisor 1 <= d < 2^31 by one multiply-high
// (Hacker's Delight, round-up method): (umulhi(n, m) + n) >> s with
// s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1.
struct FastDiv {
    uint32_t d, m, s;
};
static inline FastDiv make_div(uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    f.s = l;
    f.m = (uint32_t)((((1ull << l) - d) << 32) / d + 1);
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return (__umulhi(n, f.m) + n) >> f.s;
}

// ------------------------------------------------- persistent graph runs
// Shared by the graph engines' cooperative launches (isg_graph.cu,
// isg_cgraph.cu): a bounded grid barrier and the exchange parameters.
constexpr long long kBarrierCycles = 1ll << 34;  // ~8 s at 2 GHz

struct GraphPtParams {
    const double* betas;     // per slot
    int32_t* t2r;
    unsigned long long* ctrl;  // [0] exchange count, [1] accepted
    double* ebuf;            // [2][R]
    unsigned int* bar;       // [0] arrivals, [1] generation
    int* err;
    int64_t n_sweeps;
    uint64_t ksample0;       // sampling sweeps before this run
    int ee, me;
};

__device__ __forceinline__ bool grid_barrier(unsigned int* bar, int* err, unsigned int nblocks,
                                             long long limit = kBarrierCycles) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = bar + 1;
        const unsigned int gen = *vgen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(bar, 1u) + 1u == nblocks) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == gen) {
                if (*(volatile int*)err != 0) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > limit) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        s_ok = ok && *(volatile int*)err == 0;
    }
    __syncthreads();
    return s_ok != 0;
}


// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

}  // namespace isg

#define ISG_CK(call)                                                   \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return ::isg::cuda_fail(_e, #call);     \
    } while (0)
