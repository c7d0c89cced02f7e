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
