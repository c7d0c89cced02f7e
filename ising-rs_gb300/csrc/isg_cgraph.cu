// isg_cgraph.cu — parallel tempering of continuous spins on arbitrary graphs:
// Heisenberg O(3) with cone Metropolis and XY O(2) with single-cluster Wolff
// flips, the GPU form of the continuous-spin graph J-fitting runs.
//
// Reference path being replaced (faulknco/ising-rs):
//   src/bin/gpu_jfit.rs:414-524      run_heisenberg_jfit: one random-site
//                                    Metropolis sweep (cone of half-angle 0.5,
//                                    src/heisenberg/metropolis.rs:8-92) per
//                                    replica per sample
//   src/bin/gpu_jfit.rs:298-412      run_xy_jfit: one Wolff cluster flip
//                                    (src/xy/wolff.rs:15-78) per replica per
//                                    sample
//   src/heisenberg/mod.rs:56-74, src/xy/mod.rs:47-64
//                                    E = -J sum_bonds S.S', M = sum S
//   src/parallel_tempering.rs:5-36   replica_exchange every exchange_every
//
// GB300 form: one CTA per replica keeps the replica's spins in shared memory
// (FP32, one array per component) for a whole exchange period.
//  * O(3): colour class by colour class of a greedy proper colouring, every
//    node of a class proposes a rotation inside the cone around its spin and
//    accepts with the Metropolis rule on the local field (FP32).
//  * O(2): one Wolff cluster per sweep grown breadth-first by the whole CTA:
//    the nodes of the current level test their neighbours in parallel, a
//    shared bitmask (atomicOr) admits each node once and a shared queue holds
//    the cluster.  Each directed test (node i, adjacency slot k) has its own
//    Philox word, so the cluster is the set reachable from the seed over the
//    bonds whose words pass — the same set a sequential depth-first growth
//    with those words finds, independent of thread timing.  The reflection
//    S -> S - 2 (S.r) r and the renormalisation follow when the cluster is
//    complete.
//  * Measurement: per node the FP32 dot of its spin with its neighbour sum,
//    summed in FP64 in a fixed order (deterministic); M per component in FP64.
//
// Random stream (Philox4x32-10, key = seed; tag CGRAPH): counter
// {replica, c1, lo32(sweep), CGRAPH << 24 | field << 16 | hi16(sweep)}:
//   hot start       c1 = node, field 0xFE, sweep 0: O(3) z = 2 u0 - 1 and
//                   phi = 2 pi u1; O(2) phi = 2 pi u0 (24-bit uniforms);
//   O(3) Metropolis c1 = node, field = colour class: cos(theta) =
//                   1 - u0 (1 - cos delta), phi = 2 pi u1, accept iff dE <= 0
//                   or u2 < exp(-beta dE);
//   O(2) cluster    c1 = 0xFFFFFFFF, field 0xFD: mirror angle 2 pi u0, seed
//                   node = (w1 * n) >> 32;
//   O(2) bond test  c1 = node i, field 0xC0 + k / 4, word k % 4 for adjacency
//                   slot k of i: bond iff the projections have the same sign
//                   and u < 1 - exp(-2 beta J |p_i| |p_j|).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {

cudaError_t launch_graph_exchange(const double* energies, int32_t* r2t, int32_t* t2r,
                                  const double* betas, int R, unsigned long long* ctrl,
                                  uint64_t seed, cudaStream_t stream);

constexpr uint32_t kTagCGraph = ISG_TAG_CGRAPH;
constexpr int kCGThreads = 512;
constexpr int kCGMaxNodes = 16384;
constexpr int kCGMaxDeg = 64;
constexpr int kCGMaxReplicas = 1024;

struct CGraphParams {
    const int32_t* rowptr;   // [n+1]
    const int32_t* adj;      // [2m]
    const int32_t* order;    // nodes by colour class
    const int32_t* cstart;   // [n_classes+1]
    const int32_t* nlow;     // O(3): neighbours of lower colour, listed first in adj
    float* spins;            // [R][NC][n]
    const float* betaf;      // [slots]
    int32_t* r2t;            // [R]
    double* rec_e;           // [rows][R]
    double* rec_m;           // [rows][R][NC]
    int32_t* rec_t;          // [rows][R]
    double* last_e;          // [R] energy after the launch's last sweep
    unsigned long long* moves;  // [R] accepted rotations (O(3)) or cluster sizes (O(2))
    uint64_t seed;
    uint64_t sweep0;
    float J, cos_delta;
    int n, R, n_classes;
    int max_deg;             // largest node degree (>= 1)
    int n_sweeps;
    int measure_every, measure_phase;
    int64_t row0;
};

// Component planes of one replica's spins in shared memory.
struct Planes {
    float* x;
    float* y;
    float* z;
    __device__ __forceinline__ float* operator[](int k) const { return k == 0 ? x : k == 1 ? y : z; }
};

// Warp sum of a 64-bit int, stored in the warp's slot of slots[32].
__device__ __forceinline__ void warp_store_ll(long long v, long long* slots) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(ISG_FULL_MASK, v, o);
    if ((threadIdx.x & 31) == 0) slots[threadIdx.x >> 5] = v;
}

// Fixed point of the measurement sums: 2^40 units per spin component.  Every
// node term (|S.h| <= 64, |S_k| <= 1) converts exactly up to 2^-41, the int64
// sums are exact and independent of their order (|sum| < 2^61).
constexpr double kFixInv = 1.0 / 1099511627776.0;

// round(x 2^40) for |x| <= 64 from two 32-bit conversions (the FP32 pipe; a
// 64-bit conversion would run on the slow FP64 pipe): with h = floor(x 2^20),
// x 2^20 - h is exact, so h 2^20 + round((x 2^20 - h) 2^20) = round(x 2^40).
__device__ __forceinline__ long long fix(float x) {
    const float y = x * 1048576.0f;
    const float h = floorf(y);
    return ((long long)__float2int_rn(h) << 20) + __float2int_rn((y - h) * 1048576.0f);
}

// O(2) measurement by gathering every node's neighbour field: per-warp sums
// of sum_v S_v.h_v (twice the bond sum) and M in acc[0..2][32] (all threads
// call).
__device__ __forceinline__ void cg_measure_xy(const CGraphParams& P, const Planes& s,
                                              long long (*acc)[32]) {
    long long e = 0, m0 = 0, m1 = 0;
    for (int v = threadIdx.x; v < P.n; v += blockDim.x) {
        const int r0 = __ldg(P.rowptr + v), r1 = __ldg(P.rowptr + v + 1);
        float hx = 0.f, hy = 0.f;
        for (int j = r0; j < r1; ++j) {
            const int u = __ldg(P.adj + j);
            hx += s[0][u];
            hy += s[1][u];
        }
        const float sx = s[0][v], sy = s[1][v];
        e += fix(fmaf(sx, hx, sy * hy));
        m0 += fix(sx);
        m1 += fix(sy);
    }
    warp_store_ll(e, acc[0]);
    warp_store_ll(m0, acc[1]);
    warp_store_ll(m1, acc[2]);
}

// One cone-Metropolis sweep of an O(3) replica (spins in shared memory).  With
// `meas`, also adds sum_v S_v.h<_v (h< = the field of the lower-colour
// neighbours, final when v is updated, so every bond counts once with final
// spins) and M as per-warp sums in acc[0..3][32] before the last class's
// barrier.
__device__ __forceinline__ void cg_metropolis(const CGraphParams& P, const Planes& s, int r,
                                              uint64_t sweep, float beta, bool meas,
                                              long long (*acc)[32], unsigned long long& moves) {
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    long long pe = 0, pm0 = 0, pm1 = 0, pm2 = 0;
    for (int c = 0; c < P.n_classes; ++c) {
        const uint32_t c3 = counter_word3(kTagCGraph, (uint32_t)c, sweep);
        const int a = __ldg(P.cstart + c), b = __ldg(P.cstart + c + 1);
        for (int q = a + threadIdx.x; q < b; q += blockDim.x) {
            const int v = __ldg(P.order + q);
            const int r0 = __ldg(P.rowptr + v), r1 = __ldg(P.rowptr + v + 1);
            const int rl = r0 + __ldg(P.nlow + v);
            float l0 = 0.f, l1 = 0.f, l2 = 0.f, h0 = 0.f, h1 = 0.f, h2 = 0.f;
            for (int j = r0; j < rl; ++j) {
                const int u = __ldg(P.adj + j);
                l0 += s[0][u];
                l1 += s[1][u];
                l2 += s[2][u];
            }
            for (int j = rl; j < r1; ++j) {
                const int u = __ldg(P.adj + j);
                h0 += s[0][u];
                h1 += s[1][u];
                h2 += s[2][u];
            }
            const float hx = l0 + h0, hy = l1 + h1, hz = l2 + h2;
            const float v0 = s[0][v], v1 = s[1][v], v2 = s[2][v];
            const U4 u = philox10((uint32_t)r, (uint32_t)v, (uint32_t)sweep, c3, k0, k1);
            const float ct = 1.0f - uniform24(u.x) * (1.0f - P.cos_delta);
            const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
            float sp, cp;
            sincospif(2.0f * uniform24(u.y), &sp, &cp);
            // frame perpendicular to the spin (heisenberg/metropolis.rs:72-92)
            const float tx = fabsf(v0) < 0.9f ? 1.0f : 0.0f;
            const float ty = 1.0f - tx;
            const float ts = tx * v0 + ty * v1;
            float ux = tx - ts * v0, uy = ty - ts * v1, uz = -ts * v2;
            const float un = rsqrtf(ux * ux + uy * uy + uz * uz);
            ux *= un;
            uy *= un;
            uz *= un;
            const float wx0 = v1 * uz - v2 * uy;
            const float wy0 = v2 * ux - v0 * uz;
            const float wz0 = v0 * uy - v1 * ux;
            const float pa = st * cp, pb = st * sp;
            float w0 = pa * ux + pb * wx0 + ct * v0;
            float w1 = pa * uy + pb * wy0 + ct * v1;
            float w2 = pa * uz + pb * wz0 + ct * v2;
            const float wn = rsqrtf(w0 * w0 + w1 * w1 + w2 * w2);
            w0 *= wn;
            w1 *= wn;
            w2 *= wn;
            float dot = (w0 - v0) * hx;
            dot = fmaf(w1 - v1, hy, dot);
            dot = fmaf(w2 - v2, hz, dot);
            const float dE = -P.J * dot;
            float f0 = v0, f1 = v1, f2 = v2;
            if (dE <= 0.0f || uniform24(u.z) < expf(-beta * dE)) {
                s[0][v] = w0;
                s[1][v] = w1;
                s[2][v] = w2;
                f0 = w0;
                f1 = w1;
                f2 = w2;
                ++moves;
            }
            if (meas) {
                pe += fix(fmaf(f0, l0, fmaf(f1, l1, f2 * l2)));
                pm0 += fix(f0);
                pm1 += fix(f1);
                pm2 += fix(f2);
            }
        }
        if (meas && c == P.n_classes - 1) {
            warp_store_ll(pe, acc[0]);
            warp_store_ll(pm0, acc[1]);
            warp_store_ll(pm1, acc[2]);
            warp_store_ll(pm2, acc[3]);
        }
        __syncthreads();
    }
}

// One single-cluster Wolff flip of an O(2) replica.  Level-synchronous
// growth with one barrier per level: level L holds queue[base, base + cnt)
// and appends level L+1 after it through counter ctl[(L+1) % 3]; the counter
// of level L+2 is cleared during level L, when no thread reads or bumps it.
__device__ __forceinline__ void cg_wolff(const CGraphParams& P, const Planes& s, uint32_t* inb, int32_t* queue,
                         int* ctl, int r, uint64_t sweep, float beta) {
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const int nwords = (P.n + 31) >> 5;
    for (int w = threadIdx.x; w < nwords; w += blockDim.x) inb[w] = 0u;
    __shared__ float s_r[2];
    __syncthreads();
    if (threadIdx.x == 0) {
        const U4 u = philox10((uint32_t)r, 0xFFFFFFFFu, (uint32_t)sweep,
                              counter_word3(kTagCGraph, 0xFDu, sweep), k0, k1);
        float sp, cp;
        sincospif(2.0f * uniform24(u.x), &sp, &cp);
        s_r[0] = cp;
        s_r[1] = sp;
        const int seed_node = (int)(((uint64_t)u.y * (uint64_t)P.n) >> 32);
        inb[seed_node >> 5] = 1u << (seed_node & 31);
        queue[0] = seed_node;
        ctl[0] = 1;  // level 0: the seed
        ctl[1] = 0;
        ctl[2] = 0;
    }
    __syncthreads();
    const float twobj = 2.0f * beta * P.J;
    const float rx = s_r[0], ry = s_r[1];
    int base = 0, level = 0;
    int cnt = ctl[0];
    // a level-L node is at distance L from the seed, so there are at most n levels
    while (cnt > 0 && level < P.n) {
        int* next = &ctl[(level + 1) % 3];
        if (threadIdx.x == 0) ctl[(level + 2) % 3] = 0;
        const int end = base + cnt;
        // one (frontier node, adjacency slot) test per thread
        const int tasks = cnt * P.max_deg;
        for (int t = threadIdx.x; t < tasks; t += blockDim.x) {
            const int qo = t / P.max_deg;
            const int k = t - qo * P.max_deg;
            const int i = queue[base + qo];
            const int r0 = __ldg(P.rowptr + i);
            if (k >= __ldg(P.rowptr + i + 1) - r0) continue;
            const int j = __ldg(P.adj + r0 + k);
            const uint32_t bit = 1u << (j & 31);
            if (inb[j >> 5] & bit) continue;
            const float pi = s[0][i] * rx + s[1][i] * ry;
            const float pj = s[0][j] * rx + s[1][j] * ry;
            if (pi * pj <= 0.0f) continue;
            const float p = 1.0f - expf(-twobj * fabsf(pi) * fabsf(pj));
            const U4 u = philox10((uint32_t)r, (uint32_t)i, (uint32_t)sweep,
                                  counter_word3(kTagCGraph, 0xC0u + ((uint32_t)k >> 2), sweep), k0,
                                  k1);
            const uint32_t wk = (k & 3) == 0 ? u.x : (k & 3) == 1 ? u.y : (k & 3) == 2 ? u.z : u.w;
            if (uniform24(wk) < p) {
                const uint32_t old = atomicOr(&inb[j >> 5], bit);
                if (!(old & bit)) queue[end + atomicAdd(next, 1)] = j;
            }
        }
        __syncthreads();
        base = end;
        cnt = *next;
        ++level;
    }
    // reflect the cluster (queue[0, base)) and renormalise
    for (int q = threadIdx.x; q < base; q += blockDim.x) {
        const int i = queue[q];
        float a = s[0][i], b = s[1][i];
        const float d = a * rx + b * ry;
        a -= 2.0f * d * rx;
        b -= 2.0f * d * ry;
        const float nr = rsqrtf(a * a + b * b);
        s[0][i] = a * nr;
        s[1][i] = b * nr;
    }
    if (threadIdx.x == 0) ctl[0] = base;  // cluster size for the move counter
    __syncthreads();
}

// Running state of one replica's sweeps within a launch.
struct CGState {
    int mb;                     // slot set of the next measurement
    int64_t row;                // next record row
    unsigned long long moves;   // this thread's accepted rotations / cluster sizes
};

// n sweeps of replica r from global sweep sweep0, recording after local sweep
// k when every > 0 and k % every == phase; the energy after the last sweep
// ends up in e_last (thread 0).  A measured sweep's per-warp sums go to one
// of two alternating slot sets; thread 0 adds them after the barrier that
// follows, and the set is written again two measurements later, after
// another barrier.
template <int NC>
__device__ __forceinline__ void cg_run(const CGraphParams& P, const Planes& s, uint32_t* inb,
                                       int32_t* queue, int* ctl, long long (*s_acc)[4][32], int r,
                                       int slot, float beta, uint64_t sweep0, int n, int every,
                                       int phase, CGState& st, double& e_last) {
    for (int k = 0; k < n; ++k) {
        const uint64_t sweep = sweep0 + (uint64_t)k;
        const bool rec = every > 0 && k % every == phase;
        const bool meas = rec || k == n - 1;
        if (NC == 3) {
            cg_metropolis(P, s, r, sweep, beta, meas, s_acc[st.mb], st.moves);
        } else {
            cg_wolff(P, s, inb, queue, ctl, r, sweep, beta);
            if (threadIdx.x == 0) st.moves += (unsigned long long)ctl[0];
            if (meas) {
                cg_measure_xy(P, s, s_acc[st.mb]);
                __syncthreads();
            }
        }
        if (meas) {
            if (threadIdx.x == 0) {
                long long a[NC + 1];
#pragma unroll
                for (int c = 0; c <= NC; ++c) a[c] = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
#pragma unroll
                    for (int c = 0; c <= NC; ++c) a[c] += s_acc[st.mb][c][w];
                // O(3): each bond once; O(2): every bond from both ends
                const double bonds = (double)a[0] * kFixInv * (NC == 3 ? 1.0 : 0.5);
                const double e = -(double)P.J * bonds;
                if (rec) {
                    P.rec_e[st.row * P.R + r] = e;
#pragma unroll
                    for (int c = 0; c < NC; ++c)
                        P.rec_m[(st.row * P.R + r) * NC + c] = (double)a[1 + c] * kFixInv;
                    P.rec_t[st.row * P.R + r] = slot;
                }
                e_last = e;
            }
            st.mb ^= 1;
        }
        if (rec) ++st.row;
    }
}

// Shared-memory planes of a replica and its staging from global memory.
template <int NC>
__device__ __forceinline__ Planes cg_stage(const CGraphParams& P, float* cg_smem, int r) {
    Planes s;
    s.x = cg_smem;
    s.y = cg_smem + P.n;
    s.z = NC == 3 ? cg_smem + 2 * (size_t)P.n : cg_smem;
    const float* g = P.spins + (size_t)r * NC * P.n;
    for (int i = threadIdx.x; i < NC * P.n; i += blockDim.x) cg_smem[i] = g[i];
    __syncthreads();
    return s;
}

// Move counter (warp sums, one atomic per warp) and spins back to global.
template <int NC>
__device__ __forceinline__ void cg_finish(const CGraphParams& P, const float* cg_smem, int r,
                                          unsigned long long moves) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) moves += __shfl_down_sync(ISG_FULL_MASK, moves, o);
    if ((threadIdx.x & 31) == 0 && moves) atomicAdd(&P.moves[r], moves);
    __syncthreads();
    float* g = P.spins + (size_t)r * NC * P.n;
    for (int i = threadIdx.x; i < NC * P.n; i += blockDim.x) g[i] = cg_smem[i];
}

// n_sweeps sweeps of every replica (block = replica) between exchange points.
template <int NC>
__global__ void __launch_bounds__(kCGThreads, 1) k_cgraph_sweeps(const __grid_constant__ CGraphParams P) {
    extern __shared__ float cg_smem[];
    __shared__ long long s_acc[2][4][32];
    __shared__ int ctl[3];
    const int r = blockIdx.x;
    const Planes s = cg_stage<NC>(P, cg_smem, r);
    uint32_t* inb = reinterpret_cast<uint32_t*>(cg_smem + (size_t)NC * P.n);
    int32_t* queue = reinterpret_cast<int32_t*>(inb + ((P.n + 31) >> 5));
    const int slot = P.r2t[r];
    CGState st{0, P.row0, 0ull};
    double e = 0.0;
    cg_run<NC>(P, s, inb, queue, ctl, s_acc, r, slot, P.betaf[slot], P.sweep0, P.n_sweeps,
               P.measure_every, P.measure_phase, st, e);
    if (threadIdx.x == 0) P.last_e[r] = e;
    cg_finish<NC>(P, cg_smem, r, st.moves);
}

// A whole sampling run in one cooperative launch, as k_graph_pt: sweeps between
// exchange points, then every block publishes its energy, all meet at the
// bounded grid barrier and every block computes the same exchange pass
// (the rule of k_graph_exchange) on its own copy of the ladder.
template <int NC>
__global__ void __launch_bounds__(kCGThreads, 1)
    k_cgraph_pt(const __grid_constant__ CGraphParams P, const __grid_constant__ GraphPtParams X) {
    extern __shared__ float cg_smem[];
    __shared__ long long s_acc[2][4][32];
    __shared__ int ctl[3];
    __shared__ int s_t2r[kCGMaxReplicas];
    __shared__ int s_slot, s_acc_x;
    const int r = blockIdx.x, R = P.R;
    for (int i = threadIdx.x; i < R; i += blockDim.x) s_t2r[i] = X.t2r[i];
    const Planes s = cg_stage<NC>(P, cg_smem, r);
    uint32_t* inb = reinterpret_cast<uint32_t*>(cg_smem + (size_t)NC * P.n);
    int32_t* queue = reinterpret_cast<int32_t*>(inb + ((P.n + 31) >> 5));
    int slot = P.r2t[r];
    CGState st{0, 0, 0ull};
    unsigned long long xc = X.ctrl[0];
    int accepted = 0;
    uint64_t k = X.ksample0;
    int64_t done = 0;
    double e = 0.0;
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    while (done < X.n_sweeps) {
        const uint64_t to_x = (uint64_t)X.ee - (k % (uint64_t)X.ee);
        const int n = (int)min(to_x, (uint64_t)(X.n_sweeps - done));
        const int phase = (int)(((uint64_t)X.me - 1u - (k % (uint64_t)X.me)) % (uint64_t)X.me);
        cg_run<NC>(P, s, inb, queue, ctl, s_acc, r, slot, P.betaf[slot], P.sweep0 + (uint64_t)done,
                   n, X.me, phase, st, e);
        k += (uint64_t)n;
        done += n;
        if (k % (uint64_t)X.ee != 0) continue;
        double* eb = X.ebuf + (size_t)(xc & 1ull) * R;
        if (threadIdx.x == 0) {
            eb[r] = e;
            s_acc_x = 0;
        }
        if (!grid_barrier(X.bar, X.err, gridDim.x)) return;
        const int par = (int)(xc & 1ull);
        const uint32_t c3 = counter_word3(ISG_TAG_EXCH, 0, xc);
        for (int i = par + 2 * threadIdx.x; i + 1 < R; i += 2 * blockDim.x) {
            const int ri = s_t2r[i], rj = s_t2r[i + 1];
            const double d = __dmul_rn(__dsub_rn(X.betas[i], X.betas[i + 1]),
                                       __dsub_rn(__ldcg(eb + rj), __ldcg(eb + ri)));
            bool ok = d < 0.0;
            if (!ok) {
                const U4 u = philox10(0xFFFFFFFFu, (uint32_t)i, (uint32_t)xc, c3, k0, k1);
                ok = uniform53(u.x, u.y) < exp(-d);
            }
            if (ok) {
                s_t2r[i] = rj;
                s_t2r[i + 1] = ri;
                atomicAdd(&s_acc_x, 1);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < R; i += blockDim.x)
            if (s_t2r[i] == r) s_slot = i;
        accepted += s_acc_x;
        ++xc;
        __syncthreads();
        slot = s_slot;
    }
    if (threadIdx.x == 0) {
        P.last_e[r] = e;
        P.r2t[r] = slot;
    }
    cg_finish<NC>(P, cg_smem, r, st.moves);
    if (r == 0) {
        for (int i = threadIdx.x; i < R; i += blockDim.x) X.t2r[i] = s_t2r[i];
        if (threadIdx.x == 0) {
            X.ctrl[0] = xc;
            X.ctrl[1] += (unsigned long long)accepted;
        }
    }
}

// Hot start of every replica: [R][NC][n].
__global__ void k_cgraph_init(float* spins, int n, int R, int nc, uint64_t seed) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t c3 = counter_word3(kTagCGraph, 0xFEu, 0);
    const int64_t total = (int64_t)n * R;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / n), v = (int)(t - (int64_t)r * n);
        const U4 u = philox10((uint32_t)r, (uint32_t)v, 0u, c3, k0, k1);
        float* g = spins + (size_t)r * nc * n;
        if (nc == 3) {
            const float zz = 2.0f * uniform24(u.x) - 1.0f;
            float sp, cp;
            sincospif(2.0f * uniform24(u.y), &sp, &cp);
            const float rr = sqrtf(fmaxf(0.0f, 1.0f - zz * zz));
            g[v] = rr * cp;
            g[n + v] = rr * sp;
            g[2 * n + v] = zz;
        } else {
            float sp, cp;
            sincospif(2.0f * uniform24(u.x), &sp, &cp);
            g[v] = cp;
            g[n + v] = sp;
        }
    }
}

}  // namespace isg

using namespace isg;

struct isg_cgraph {
    int device = 0;
    int n = 0, m = 0, R = 0, nc = 3, n_classes = 0, max_deg = 1;
    uint64_t seed = 0;
    double J = 1.0, delta = 0.5;
    bool temps_set = false;
    uint64_t gsweep = 0;
    uint64_t ksample = 0;
    size_t smem = 0;
    int32_t* d_rowptr = nullptr;
    int32_t* d_adj = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_cstart = nullptr;
    int32_t* d_nlow = nullptr;
    float* d_spins = nullptr;
    float* d_betaf = nullptr;
    double* d_betas = nullptr;
    int32_t* d_r2t = nullptr;
    int32_t* d_t2r = nullptr;
    double* d_last_e = nullptr;
    unsigned long long* d_moves = nullptr;
    // persistent runs (k_cgraph_pt): energy buffers, barrier, error flag
    double* d_ebuf = nullptr;
    unsigned int* d_bar = nullptr;
    int* d_err = nullptr;
    bool coop = false;         // all replicas can be resident at once
    unsigned long long* d_ctrl = nullptr;  // [0] exchange count, [1] accepted
    double* d_rec_e = nullptr;
    double* d_rec_m = nullptr;
    int32_t* d_rec_t = nullptr;
    int64_t rec_cap = 0;
    cudaStream_t stream = nullptr;
};

namespace {

int cg_destroy(isg_cgraph* H) {
    if (!H) return ISG_OK;
    cudaSetDevice(H->device);
    if (H->stream) cudaStreamSynchronize(H->stream);
    cudaFree(H->d_rowptr);
    cudaFree(H->d_adj);
    cudaFree(H->d_order);
    cudaFree(H->d_cstart);
    cudaFree(H->d_nlow);
    cudaFree(H->d_spins);
    cudaFree(H->d_betaf);
    cudaFree(H->d_betas);
    cudaFree(H->d_r2t);
    cudaFree(H->d_t2r);
    cudaFree(H->d_last_e);
    cudaFree(H->d_moves);
    cudaFree(H->d_ebuf);
    cudaFree(H->d_bar);
    cudaFree(H->d_err);
    cudaFree(H->d_ctrl);
    cudaFree(H->d_rec_e);
    cudaFree(H->d_rec_m);
    cudaFree(H->d_rec_t);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
    return ISG_OK;
}

CGraphParams cg_params(isg_cgraph* H, int n_sweeps, int every, int phase, int64_t row0) {
    CGraphParams P{};
    P.rowptr = H->d_rowptr;
    P.adj = H->d_adj;
    P.order = H->d_order;
    P.cstart = H->d_cstart;
    P.nlow = H->d_nlow;
    P.spins = H->d_spins;
    P.betaf = H->d_betaf;
    P.r2t = H->d_r2t;
    P.rec_e = H->d_rec_e;
    P.rec_m = H->d_rec_m;
    P.rec_t = H->d_rec_t;
    P.last_e = H->d_last_e;
    P.moves = H->d_moves;
    P.seed = H->seed;
    P.sweep0 = H->gsweep;
    P.J = (float)H->J;
    P.cos_delta = (float)std::cos(H->delta);
    P.n = H->n;
    P.R = H->R;
    P.n_classes = H->n_classes;
    P.max_deg = H->max_deg;
    P.n_sweeps = n_sweeps;
    P.measure_every = every;
    P.measure_phase = phase;
    P.row0 = row0;
    return P;
}

int cg_launch(isg_cgraph* H, int n_sweeps, int every, int phase, int64_t row0) {
    const CGraphParams P = cg_params(H, n_sweeps, every, phase, row0);
    if (H->nc == 3)
        k_cgraph_sweeps<3><<<H->R, kCGThreads, H->smem, H->stream>>>(P);
    else
        k_cgraph_sweeps<2><<<H->R, kCGThreads, H->smem, H->stream>>>(P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_cgraph_sweeps");
    H->gsweep += (uint64_t)n_sweeps;
    return ISG_OK;
}

}  // namespace

extern "C" {

int isg_cgraph_create(isg_cgraph** out, int n_nodes, const int32_t* edges, int n_edges,
                      int replicas, int n_comp, uint64_t seed) {
    if (!out) return fail(ISG_ERR_ARG, "isg_cgraph_create: out is NULL");
    *out = nullptr;
    if (n_comp != 2 && n_comp != 3)
        return fail(ISG_ERR_ARG, "isg_cgraph_create: n_comp must be 2 (XY) or 3 (Heisenberg)");
    if (n_nodes < 1 || n_nodes > kCGMaxNodes)
        return fail(ISG_ERR_ARG, "isg_cgraph_create: n_nodes must be 1..16384");
    if (n_edges < 0 || (n_edges > 0 && !edges))
        return fail(ISG_ERR_ARG, "isg_cgraph_create: bad edge list");
    if (replicas < 1 || replicas > kCGMaxReplicas)
        return fail(ISG_ERR_ARG, "isg_cgraph_create: replicas must be 1..1024");
    std::vector<int> deg(n_nodes, 0);
    for (int e = 0; e < n_edges; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || a >= n_nodes || b >= n_nodes)
            return fail(ISG_ERR_ARG, "isg_cgraph_create: edge " + std::to_string(e) +
                                         " names a node outside 0.." +
                                         std::to_string(n_nodes - 1));
        if (a == b)
            return fail(ISG_ERR_ARG, "isg_cgraph_create: self-loop at node " + std::to_string(a));
        ++deg[a];
        ++deg[b];
    }
    for (int v = 0; v < n_nodes; ++v)
        if (deg[v] > kCGMaxDeg)
            return fail(ISG_ERR_UNSUPPORTED, "isg_cgraph_create: node " + std::to_string(v) +
                                                 " has degree " + std::to_string(deg[v]) +
                                                 " (at most 64)");
    std::vector<int32_t> rowptr(n_nodes + 1, 0), adj(2 * (size_t)n_edges);
    for (int v = 0; v < n_nodes; ++v) rowptr[v + 1] = rowptr[v] + deg[v];
    std::vector<int32_t> fillp(rowptr.begin(), rowptr.end() - 1);
    for (int e = 0; e < n_edges; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        adj[fillp[a]++] = b;
        adj[fillp[b]++] = a;
    }
    // greedy proper colouring in node order
    std::vector<int> col(n_nodes, -1);
    std::vector<char> used(kCGMaxDeg + 2, 0);
    int ncol = 0;
    for (int v = 0; v < n_nodes; ++v) {
        std::fill(used.begin(), used.end(), 0);
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
            if (col[adj[j]] >= 0) used[col[adj[j]]] = 1;
        int c = 0;
        while (used[c]) ++c;
        col[v] = c;
        ncol = std::max(ncol, c + 1);
    }
    // O(3): each node's lower-colour neighbours first (stable), counted in nlow
    std::vector<int32_t> nlow(n_nodes, 0);
    if (n_comp == 3) {
        std::vector<int32_t> tmp;
        for (int v = 0; v < n_nodes; ++v) {
            tmp.clear();
            for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
                if (col[adj[j]] < col[v]) tmp.push_back(adj[j]);
            nlow[v] = (int32_t)tmp.size();
            for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
                if (col[adj[j]] > col[v]) tmp.push_back(adj[j]);
            std::copy(tmp.begin(), tmp.end(), adj.begin() + rowptr[v]);
        }
    }
    std::vector<int32_t> cstart(ncol + 1, 0), order(n_nodes);
    for (int v = 0; v < n_nodes; ++v) ++cstart[col[v] + 1];
    for (int c = 0; c < ncol; ++c) cstart[c + 1] += cstart[c];
    std::vector<int32_t> fillc(cstart.begin(), cstart.end() - 1);
    for (int v = 0; v < n_nodes; ++v) order[fillc[col[v]]++] = v;

    isg_cgraph* H = new (std::nothrow) isg_cgraph();
    if (!H) return fail(ISG_ERR_ARG, "isg_cgraph_create: out of host memory");
    cudaGetDevice(&H->device);
    H->n = n_nodes;
    H->m = n_edges;
    H->R = replicas;
    H->nc = n_comp;
    H->seed = seed;
    H->n_classes = ncol;
    H->max_deg = std::max(1, *std::max_element(deg.begin(), deg.end()));
    // spins (+ cluster bitmask and queue for O(2)) in dynamic shared memory
    H->smem = sizeof(float) * (size_t)n_comp * n_nodes;
    if (n_comp == 2) H->smem += sizeof(uint32_t) * ((n_nodes + 31) / 32) + sizeof(int32_t) * n_nodes;
    cudaError_t e;
#define CGALLOC(ptr, bytes)                                            \
    e = cudaMalloc((void**)&(ptr), std::max<size_t>(8, (bytes)));      \
    if (e != cudaSuccess) {                                            \
        cg_destroy(H);                                                 \
        return cuda_fail(e, "cudaMalloc");                             \
    }
    CGALLOC(H->d_rowptr, sizeof(int32_t) * (n_nodes + 1));
    CGALLOC(H->d_adj, sizeof(int32_t) * adj.size());
    CGALLOC(H->d_order, sizeof(int32_t) * n_nodes);
    CGALLOC(H->d_cstart, sizeof(int32_t) * (ncol + 1));
    CGALLOC(H->d_nlow, sizeof(int32_t) * n_nodes);
    CGALLOC(H->d_spins, sizeof(float) * (size_t)n_comp * n_nodes * replicas);
    CGALLOC(H->d_betaf, sizeof(float) * replicas);
    CGALLOC(H->d_betas, sizeof(double) * replicas);
    CGALLOC(H->d_r2t, sizeof(int32_t) * replicas);
    CGALLOC(H->d_t2r, sizeof(int32_t) * replicas);
    CGALLOC(H->d_last_e, sizeof(double) * replicas);
    CGALLOC(H->d_moves, sizeof(unsigned long long) * replicas);
    CGALLOC(H->d_ebuf, sizeof(double) * 2 * replicas);
    CGALLOC(H->d_bar, sizeof(unsigned int) * 2);
    CGALLOC(H->d_err, sizeof(int));
    CGALLOC(H->d_ctrl, sizeof(unsigned long long) * 2);
#undef CGALLOC
    e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cg_destroy(H);
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    if (H->smem > 48 * 1024) {
        const int a = cudaFuncAttributeMaxDynamicSharedMemorySize;
        e = n_comp == 3 ? cudaFuncSetAttribute(k_cgraph_sweeps<3>, (cudaFuncAttribute)a,
                                               (int)H->smem)
                        : cudaFuncSetAttribute(k_cgraph_sweeps<2>, (cudaFuncAttribute)a,
                                               (int)H->smem);
        if (e == cudaSuccess)
            e = n_comp == 3 ? cudaFuncSetAttribute(k_cgraph_pt<3>, (cudaFuncAttribute)a, (int)H->smem)
                            : cudaFuncSetAttribute(k_cgraph_pt<2>, (cudaFuncAttribute)a, (int)H->smem);
        if (e != cudaSuccess) {
            cg_destroy(H);
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    {
        // a persistent run needs every replica resident at once
        int coop_attr = 0, sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&coop_attr, cudaDevAttrCooperativeLaunch, H->device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device);
        const cudaError_t oe =
            n_comp == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgraph_pt<3>,
                                                                        kCGThreads, H->smem)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cgraph_pt<2>,
                                                                        kCGThreads, H->smem);
        if (oe != cudaSuccess) per_sm = 0;
        cudaGetLastError();
        H->coop = coop_attr && (int64_t)per_sm * sms >= replicas;
    }
    std::vector<int32_t> ident(replicas);
    for (int r = 0; r < replicas; ++r) ident[r] = r;
#define CGCK(call)                                                     \
    e = (call);                                                        \
    if (e != cudaSuccess) {                                            \
        cg_destroy(H);                                                 \
        return cuda_fail(e, #call);                                    \
    }
    CGCK(cudaMemcpyAsync(H->d_rowptr, rowptr.data(), sizeof(int32_t) * rowptr.size(),
                         cudaMemcpyHostToDevice, H->stream));
    if (!adj.empty())
        CGCK(cudaMemcpyAsync(H->d_adj, adj.data(), sizeof(int32_t) * adj.size(),
                             cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemcpyAsync(H->d_order, order.data(), sizeof(int32_t) * n_nodes,
                         cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemcpyAsync(H->d_cstart, cstart.data(), sizeof(int32_t) * cstart.size(),
                         cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemcpyAsync(H->d_nlow, nlow.data(), sizeof(int32_t) * n_nodes,
                         cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * replicas,
                         cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * replicas,
                         cudaMemcpyHostToDevice, H->stream));
    CGCK(cudaMemsetAsync(H->d_ctrl, 0, sizeof(unsigned long long) * 2, H->stream));
    CGCK(cudaMemsetAsync(H->d_moves, 0, sizeof(unsigned long long) * replicas, H->stream));
    CGCK(cudaMemsetAsync(H->d_bar, 0, sizeof(unsigned int) * 2, H->stream));
    CGCK(cudaMemsetAsync(H->d_err, 0, sizeof(int), H->stream));
    k_cgraph_init<<<std::max(1, std::min(1024, (n_nodes * replicas + 255) / 256)), 256, 0,
                    H->stream>>>(H->d_spins, n_nodes, replicas, n_comp, seed);
    CGCK(cudaGetLastError());
    CGCK(cudaStreamSynchronize(H->stream));
#undef CGCK
    *out = H;
    return ISG_OK;
}

int isg_cgraph_destroy(isg_cgraph* h) { return cg_destroy(h); }

int isg_cgraph_num_colours(isg_cgraph* h, int* n) {
    if (!h || !n) return fail(ISG_ERR_ARG, "isg_cgraph_num_colours: NULL argument");
    *n = h->n_classes;
    return ISG_OK;
}

int isg_cgraph_set_temperatures(isg_cgraph* h, const double* temps, double J) {
    if (!h || !temps) return fail(ISG_ERR_ARG, "isg_cgraph_set_temperatures: NULL argument");
    if (!std::isfinite(J)) return fail(ISG_ERR_ARG, "isg_cgraph_set_temperatures: J must be finite");
    cudaSetDevice(h->device);
    const int R = h->R;
    std::vector<double> betas(R);
    std::vector<float> betaf(R);
    for (int t = 0; t < R; ++t) {
        if (!(temps[t] > 0.0) || !std::isfinite(temps[t]))
            return fail(ISG_ERR_ARG, "isg_cgraph_set_temperatures: temperatures must be positive");
        betas[t] = 1.0 / temps[t];
        betaf[t] = (float)betas[t];
    }
    std::vector<int32_t> ident(R);
    for (int r = 0; r < R; ++r) ident[r] = r;
    ISG_CK(cudaMemcpyAsync(h->d_betas, betas.data(), sizeof(double) * R, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaMemcpyAsync(h->d_betaf, betaf.data(), sizeof(float) * R, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaMemcpyAsync(h->d_r2t, ident.data(), sizeof(int32_t) * R, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaMemcpyAsync(h->d_t2r, ident.data(), sizeof(int32_t) * R, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    h->J = J;
    h->temps_set = true;
    return ISG_OK;
}

int isg_cgraph_set_delta(isg_cgraph* h, double delta) {
    if (!h) return fail(ISG_ERR_ARG, "isg_cgraph_set_delta: NULL handle");
    if (!(delta > 0.0) || !(delta <= 3.141592653589793))
        return fail(ISG_ERR_ARG, "isg_cgraph_set_delta: delta must be in (0, pi]");
    h->delta = delta;
    return ISG_OK;
}

int isg_cgraph_step(isg_cgraph* h, int64_t n_sweeps) {
    if (!h) return fail(ISG_ERR_ARG, "isg_cgraph_step: NULL handle");
    if (!h->temps_set) return fail(ISG_ERR_STATE, "isg_cgraph_step: temperatures not set");
    if (n_sweeps < 0) return fail(ISG_ERR_ARG, "isg_cgraph_step: negative sweep count");
    cudaSetDevice(h->device);
    for (int64_t done = 0; done < n_sweeps;) {
        const int n = (int)std::min<int64_t>(n_sweeps - done, 1 << 20);
        int rc = cg_launch(h, n, 0, 0, 0);
        if (rc) return rc;
        done += n;
    }
    return ISG_OK;
}

int isg_cgraph_reset_sampling(isg_cgraph* h) {
    if (!h) return fail(ISG_ERR_ARG, "isg_cgraph_reset_sampling: NULL handle");
    cudaSetDevice(h->device);
    ISG_CK(cudaMemsetAsync(h->d_ctrl, 0, sizeof(unsigned long long) * 2, h->stream));
    ISG_CK(cudaMemsetAsync(h->d_moves, 0, sizeof(unsigned long long) * h->R, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    h->ksample = 0;
    return ISG_OK;
}

int isg_cgraph_pt_run(isg_cgraph* h, int64_t n_sweeps, int exchange_every, int measure_every,
                      int32_t* tslot, double* e_rec, double* m_rec, int64_t max_records,
                      int64_t* n_records) {
    if (!h) return fail(ISG_ERR_ARG, "isg_cgraph_pt_run: NULL handle");
    if (!h->temps_set) return fail(ISG_ERR_STATE, "isg_cgraph_pt_run: temperatures not set");
    if (n_sweeps < 0 || exchange_every < 1 || measure_every < 1)
        return fail(ISG_ERR_ARG, "isg_cgraph_pt_run: need n_sweeps >= 0, exchange_every >= 1, "
                                 "measure_every >= 1");
    const uint64_t k0 = h->ksample;
    const int64_t need = (int64_t)((k0 + (uint64_t)n_sweeps) / (uint64_t)measure_every -
                                   k0 / (uint64_t)measure_every);
    if (need > 0 && (!tslot || !e_rec || !m_rec || max_records < need))
        return fail(ISG_ERR_ARG, "isg_cgraph_pt_run: record arrays hold " +
                                     std::to_string(max_records) + " rows, " +
                                     std::to_string(need) + " needed");
    cudaSetDevice(h->device);
    if (need > h->rec_cap) {
        cudaFree(h->d_rec_e);
        cudaFree(h->d_rec_m);
        cudaFree(h->d_rec_t);
        h->d_rec_e = h->d_rec_m = nullptr;
        h->d_rec_t = nullptr;
        h->rec_cap = 0;
        ISG_CK(cudaMalloc((void**)&h->d_rec_e, sizeof(double) * need * h->R));
        ISG_CK(cudaMalloc((void**)&h->d_rec_m, sizeof(double) * need * h->R * h->nc));
        ISG_CK(cudaMalloc((void**)&h->d_rec_t, sizeof(int32_t) * need * h->R));
        h->rec_cap = need;
    }
    int64_t done = 0, row = 0;
    if (h->coop && exchange_every <= 100000 && n_sweeps > 0) {
        // the whole run in one cooperative launch (k_cgraph_pt)
        CGraphParams P = cg_params(h, 0, measure_every, 0, 0);
        GraphPtParams X{};
        X.betas = h->d_betas;
        X.t2r = h->d_t2r;
        X.ctrl = h->d_ctrl;
        X.ebuf = h->d_ebuf;
        X.bar = h->d_bar;
        X.err = h->d_err;
        X.n_sweeps = n_sweeps;
        X.ksample0 = h->ksample;
        X.ee = exchange_every;
        X.me = measure_every;
        void* args[] = {&P, &X};
        const void* fn = h->nc == 3 ? (const void*)k_cgraph_pt<3> : (const void*)k_cgraph_pt<2>;
        ISG_CK(cudaLaunchCooperativeKernel(fn, dim3(h->R), dim3(kCGThreads), args, h->smem,
                                           h->stream));
        int err = 0;
        ISG_CK(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        ISG_CK(cudaStreamSynchronize(h->stream));
        if (err)
            return fail(ISG_ERR_TIMEOUT, "isg_cgraph_pt_run: a replica did not reach the exchange "
                                         "barrier in time");
        h->gsweep += (uint64_t)n_sweeps;
        h->ksample += (uint64_t)n_sweeps;
        done = n_sweeps;
        row = need;
    }
    while (done < n_sweeps) {
        const uint64_t k = h->ksample;
        const uint64_t to_x = (uint64_t)exchange_every - (k % (uint64_t)exchange_every);
        const int n = (int)std::min<uint64_t>(to_x, (uint64_t)(n_sweeps - done));
        const int phase = (int)(((uint64_t)measure_every - 1u - (k % (uint64_t)measure_every)) %
                                (uint64_t)measure_every);
        int rc = cg_launch(h, n, measure_every, phase, row);
        if (rc) return rc;
        if (n > phase) row += (n - 1 - phase) / measure_every + 1;
        h->ksample += (uint64_t)n;
        done += n;
        if (h->ksample % (uint64_t)exchange_every == 0) {
            cudaError_t e = launch_graph_exchange(h->d_last_e, h->d_r2t, h->d_t2r, h->d_betas,
                                                  h->R, h->d_ctrl, h->seed, h->stream);
            if (e != cudaSuccess) return cuda_fail(e, "k_graph_exchange");
        }
    }
    if (n_records) *n_records = row;
    if (row > 0) {
        ISG_CK(cudaMemcpyAsync(tslot, h->d_rec_t, sizeof(int32_t) * row * h->R,
                               cudaMemcpyDeviceToHost, h->stream));
        ISG_CK(cudaMemcpyAsync(e_rec, h->d_rec_e, sizeof(double) * row * h->R,
                               cudaMemcpyDeviceToHost, h->stream));
        ISG_CK(cudaMemcpyAsync(m_rec, h->d_rec_m, sizeof(double) * row * h->R * h->nc,
                               cudaMemcpyDeviceToHost, h->stream));
    }
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

int isg_cgraph_get_accepted(isg_cgraph* h, int64_t* accepted) {
    if (!h || !accepted) return fail(ISG_ERR_ARG, "isg_cgraph_get_accepted: NULL argument");
    cudaSetDevice(h->device);
    unsigned long long c[2];
    ISG_CK(cudaMemcpyAsync(c, h->d_ctrl, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    *accepted = (int64_t)c[1];
    return ISG_OK;
}

int isg_cgraph_get_moves(isg_cgraph* h, int64_t* moves) {
    if (!h || !moves) return fail(ISG_ERR_ARG, "isg_cgraph_get_moves: NULL argument");
    cudaSetDevice(h->device);
    std::vector<unsigned long long> d(h->R);
    ISG_CK(cudaMemcpyAsync(d.data(), h->d_moves, sizeof(unsigned long long) * h->R,
                           cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    for (int r = 0; r < h->R; ++r) moves[r] = (int64_t)d[r];
    return ISG_OK;
}

int isg_cgraph_get_spins(isg_cgraph* h, int replica, float* out) {
    if (!h || !out || replica < 0 || replica >= h->R)
        return fail(ISG_ERR_ARG, "isg_cgraph_get_spins: bad argument");
    cudaSetDevice(h->device);
    const size_t cnt = (size_t)h->nc * h->n;
    std::vector<float> d(cnt);
    ISG_CK(cudaMemcpyAsync(d.data(), h->d_spins + (size_t)replica * cnt, sizeof(float) * cnt,
                           cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    for (int v = 0; v < h->n; ++v)
        for (int k = 0; k < h->nc; ++k) out[(size_t)v * h->nc + k] = d[(size_t)k * h->n + v];
    return ISG_OK;
}

int isg_cgraph_set_spins(isg_cgraph* h, int replica, const float* in) {
    if (!h || !in || replica < 0 || replica >= h->R)
        return fail(ISG_ERR_ARG, "isg_cgraph_set_spins: bad argument");
    cudaSetDevice(h->device);
    const size_t cnt = (size_t)h->nc * h->n;
    std::vector<float> d(cnt);
    for (int v = 0; v < h->n; ++v)
        for (int k = 0; k < h->nc; ++k) d[(size_t)k * h->n + v] = in[(size_t)v * h->nc + k];
    ISG_CK(cudaMemcpyAsync(h->d_spins + (size_t)replica * cnt, d.data(), sizeof(float) * cnt,
                           cudaMemcpyHostToDevice, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

int isg_cgraph_get_r2t(isg_cgraph* h, int32_t* r2t) {
    if (!h || !r2t) return fail(ISG_ERR_ARG, "isg_cgraph_get_r2t: NULL argument");
    cudaSetDevice(h->device);
    ISG_CK(cudaMemcpyAsync(r2t, h->d_r2t, sizeof(int32_t) * h->R, cudaMemcpyDeviceToHost,
                           h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

int isg_cgraph_get_sweep(isg_cgraph* h, uint64_t* sweep) {
    if (!h || !sweep) return fail(ISG_ERR_ARG, "isg_cgraph_get_sweep: NULL argument");
    *sweep = h->gsweep;
    return ISG_OK;
}

}  // extern "C"
