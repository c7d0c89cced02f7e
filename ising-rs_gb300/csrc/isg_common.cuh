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

// Philox4x32-10 of counter {uid, w, c2, c3} with the warp-uniform part of the
// first three rounds (everything that does not depend on w) computed once per
// replica.  Products are formed as 64-bit values (one wide multiply each).
struct PhiloxPre {
    uint32_t x0, x2, x3, hi02, lo02;
};

__device__ __forceinline__ uint64_t mulw(uint32_t a, uint32_t b) { return (uint64_t)a * b; }

__device__ __forceinline__ PhiloxPre philox_pre(uint32_t uid, uint32_t c2, uint32_t c3,
                                                uint32_t k0, uint32_t k1) {
    PhiloxPre p;
    // round 0: M0*uid and M1*c2 are uniform
    const uint64_t p0 = mulw(kPhiloxM0, uid), p1 = mulw(kPhiloxM1, c2);
    p.x0 = (uint32_t)(p1 >> 32) ^ k0;  // a0 = x0 ^ w
    const uint32_t a1 = (uint32_t)p1;
    const uint32_t a2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t a3 = (uint32_t)p0;
    // round 1 (keys + W): M1*a2 uniform
    const uint64_t q1 = mulw(kPhiloxM1, a2);
    const uint32_t b0 = (uint32_t)(q1 >> 32) ^ a1 ^ (k0 + kPhiloxW0);
    const uint32_t b1 = (uint32_t)q1;
    p.x2 = a3 ^ (k1 + kPhiloxW1);  // b2 = hi(M0*a0) ^ x2, b3 = lo(M0*a0)
    // round 2 (keys + 2W): M0*b0 uniform
    const uint64_t q0 = mulw(kPhiloxM0, b0);
    p.hi02 = (uint32_t)(q0 >> 32) ^ (k1 + 2u * kPhiloxW1);  // c2 = b3 ^ hi02
    p.lo02 = (uint32_t)q0;                                  // c3
    p.x3 = b1 ^ (k0 + 2u * kPhiloxW0);                      // c0 = hi(M1*b2) ^ x3
    return p;
}

// P: any parameter block with the round keys rk0[r] = k0 + r W0, rk1[r] =
// k1 + r W1 (kernel parameters: constant-bank operands).
template <class PP>
__device__ __forceinline__ U4 philox_w(const PhiloxPre& p, const PP& P, uint32_t w) {
    const uint32_t a0 = p.x0 ^ w;
    const uint64_t r1 = mulw(kPhiloxM0, a0);
    const uint32_t b2 = (uint32_t)(r1 >> 32) ^ p.x2;
    const uint32_t b3 = (uint32_t)r1;
    const uint64_t r2 = mulw(kPhiloxM1, b2);
    uint32_t c0 = (uint32_t)(r2 >> 32) ^ p.x3;
    uint32_t c1 = (uint32_t)r2;
    uint32_t c2 = b3 ^ p.hi02;
    uint32_t c3 = p.lo02;
#pragma unroll
    for (int r = 3; r < 10; ++r) {
        const uint64_t m0 = mulw(kPhiloxM0, c0), m1 = mulw(kPhiloxM1, c2);
        c0 = (uint32_t)(m1 >> 32) ^ c1 ^ P.rk0[r];
        c1 = (uint32_t)m1;
        c2 = (uint32_t)(m0 >> 32) ^ c3 ^ P.rk1[r];
        c3 = (uint32_t)m0;
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
