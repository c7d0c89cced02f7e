// isg_graph.cu — Ising parallel tempering on arbitrary graphs (crystal graphs
// such as BCC and FCC, diluted lattices): the GPU form of the graph J-fitting
// runs.
//
// Reference path being replaced (faulknco/ising-rs):
//   src/bin/gpu_jfit.rs:172-297   run_ising_jfit: R replicas of a graph, one
//                                 random-site Metropolis sweep per replica per
//                                 sample on the host, E and M every sweep,
//                                 replica exchange every exchange_every sweeps
//   src/graph.rs:4-153            GraphDef (node count + edge list)
//   src/parallel_tempering.rs:5-36 replica_exchange
//
// GB300 form: one CTA per replica holds the replica's spins in shared memory
// for a whole exchange period; the sites are updated colour class by colour
// class of a greedy proper colouring (no two neighbours share a class, so a
// class updates in parallel), the neighbours come from a CSR adjacency in
// global memory (read-only, L1/L2 resident), and the acceptance is a uint32
// threshold indexed by (own down bit, degree, down neighbours).  The exchange
// pass runs on the device with the rule of the lattice engine.
//
// Random stream (Philox4x32-10, key = seed): sweep updates use counter
// {replica, node >> 2, lo32(sweep), GRAPH << 24 | class << 16 | hi16(sweep)},
// word node & 3; the hot start uses class 0xFE and sweep 0 (spin -1 iff the
// word's top bit is set); exchanges use counter {0xFFFFFFFF, pair index,
// lo32(count), EXCH << 24 | hi16(count)} with u = ((w0 << 32 | w1) >> 11) 2^-53.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {

constexpr int kGMaxDeg = 12;
constexpr int kGTab = 2 * (kGMaxDeg + 1) * (kGMaxDeg + 1);  // own x degree x n_down
constexpr int kGThreads = 512;
constexpr int kGMaxNodes = 65536;
constexpr int kGMaxReplicas = 1024;

struct GraphParams {
    const int32_t* rowptr;   // [n+1]
    const int32_t* adj;      // [2m]
    const int32_t* order;    // nodes by colour class, [n]
    const int32_t* cstart;   // class starts in `order`, [n_classes+1]
    uint8_t* spins;          // [R][n] down bits
    const uint32_t* thr;     // [slots][kGTab]
    int32_t* r2t;            // [R]
    long long* rec_b;        // [rows][R] bond sums (one record per measured sweep)
    long long* rec_m;
    int32_t* rec_t;
    double* last_e;          // [R] energy -J * bond after the launch's last sweep
    long long* last_bm;      // [R][2] bond sum and magnetisation after the last sweep
    int bm_known;            // last_bm holds the current state (else measure first)
    double J;
    uint64_t seed;
    uint64_t sweep0;         // global sweep of the launch's first sweep
    int n, R, n_classes;
    int n_sweeps;
    int measure_every, measure_phase;  // record after sweep k iff k % every == phase
    int64_t row0;            // record row of the first measured sweep
};

// Block sums of two ints in one pass (valid in thread 0); red holds 64 ints.
__device__ __forceinline__ void g_block_sum2(int& a, int& b, int* red) {
    a = __reduce_add_sync(ISG_FULL_MASK, a);
    b = __reduce_add_sync(ISG_FULL_MASK, b);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        red[w] = a;
        red[32 + w] = b;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = threadIdx.x < (blockDim.x >> 5);
        a = __reduce_add_sync(ISG_FULL_MASK, in ? red[threadIdx.x] : 0);
        b = __reduce_add_sync(ISG_FULL_MASK, in ? red[32 + threadIdx.x] : 0);
    }
}

// Bond sum sum_edges s_u s_v = (1/2) sum_v s_v (deg_v - 2 n_down(v)) and
// magnetisation of the spins in shared memory.
__device__ __forceinline__ void g_measure(const GraphParams& P, const uint8_t* sp, int* red,
                                          long long& bond, long long& mag) {
    int b = 0, m = 0;
    for (int v = threadIdx.x; v < P.n; v += blockDim.x) {
        const int r0 = __ldg(P.rowptr + v), r1 = __ldg(P.rowptr + v + 1);
        int nd = 0;
        for (int j = r0; j < r1; ++j) nd += sp[__ldg(P.adj + j)];
        const int s = 1 - 2 * (int)sp[v];
        b += s * ((r1 - r0) - 2 * nd);
        m += s;
    }
    g_block_sum2(b, m, red);
    bond = b / 2;
    mag = m;
}

// Warp sum of a 64-bit int, stored in the warp's slot of slots[32].
__device__ __forceinline__ void g_warp_store(long long v, long long* slots) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(ISG_FULL_MASK, v, o);
    if ((threadIdx.x & 31) == 0) slots[threadIdx.x >> 5] = v;
}

// Running bond sum / magnetisation of one replica during a launch: the values
// at the launch start (thread 0) and every thread's exact integer change since
// (-2 s (deg - 2 n_down) and -2 s per flip: the nodes of a class share no edge,
// so the changes of one class add up).
struct GState {
    long long bond0, mag0, db, dm;
    int mb;       // slot set of the next measurement
    int64_t row;  // next record row
};

// n sweeps of replica r (spins in shared memory) from global sweep sweep0,
// recording after local sweep k when every > 0 and k % every == phase.  The
// bond sum and magnetisation after the last sweep end up in bb, mm (thread 0).
// A measurement costs one warp reduction per warp before the last class's
// barrier (each warp stores its sum in its slot of one of two alternating
// slot sets) and thread 0 adds the slots after it; a slot set is written again
// two measurements later, after another barrier.
__device__ __forceinline__ void graph_run(const GraphParams& P, int r, int slot, uint8_t* g_sp,
                                          const uint32_t* s_tab, long long (*s_acc)[2][32],
                                          uint64_t sweep0, int n, int every, int phase, GState& st,
                                          long long& bb, long long& mm) {
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const int last_class = P.n_classes - 1;
    for (int k = 0; k < n; ++k) {
        const uint64_t sweep = sweep0 + (uint64_t)k;
        const bool rec = every > 0 && k % every == phase;
        const bool meas = rec || k == n - 1;
        for (int c = 0; c < P.n_classes; ++c) {
            const uint32_t c3 = counter_word3(ISG_TAG_GRAPH, (uint32_t)c, sweep);
            const int a = __ldg(P.cstart + c), b = __ldg(P.cstart + c + 1);
            for (int q = a + threadIdx.x; q < b; q += blockDim.x) {
                const int v = __ldg(P.order + q);
                const int r0 = __ldg(P.rowptr + v), r1 = __ldg(P.rowptr + v + 1);
                int nd = 0;
                for (int j = r0; j < r1; ++j) nd += g_sp[__ldg(P.adj + j)];
                const int d = g_sp[v];
                const uint32_t th = s_tab[(d * (kGMaxDeg + 1) + (r1 - r0)) * (kGMaxDeg + 1) + nd];
                const U4 u = philox10((uint32_t)r, (uint32_t)v >> 2, (uint32_t)sweep, c3, k0, k1);
                const uint32_t jv = (uint32_t)v & 3u;
                const uint32_t uw = jv == 0 ? u.x : jv == 1 ? u.y : jv == 2 ? u.z : u.w;
                if (uw <= th) {
                    g_sp[v] = (uint8_t)(d ^ 1);
                    const int s_old = 1 - 2 * d;
                    st.db -= 2 * s_old * ((r1 - r0) - 2 * nd);
                    st.dm -= 2 * s_old;
                }
            }
            if (meas && c == last_class) {
                g_warp_store(st.db, s_acc[st.mb][0]);
                g_warp_store(st.dm, s_acc[st.mb][1]);
            }
            __syncthreads();
        }
        if (meas) {
            if (threadIdx.x == 0) {
                long long b2 = st.bond0, m2 = st.mag0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                    b2 += s_acc[st.mb][0][w];
                    m2 += s_acc[st.mb][1][w];
                }
                if (rec) {
                    P.rec_b[st.row * P.R + r] = b2;
                    P.rec_m[st.row * P.R + r] = m2;
                    P.rec_t[st.row * P.R + r] = slot;
                }
                bb = b2;
                mm = m2;
            }
            st.mb ^= 1;
        }
        if (rec) ++st.row;
    }
}

// Stage replica r's spins and threshold table; the starting bond sum and
// magnetisation come from the previous launch or one measurement.
__device__ __forceinline__ void graph_stage(const GraphParams& P, int r, int slot, uint8_t* g_sp,
                                            uint32_t* s_tab, int* red, GState& st) {
    const uint8_t* spins = P.spins + (size_t)r * P.n;
    for (int v = threadIdx.x; v < P.n; v += blockDim.x) g_sp[v] = spins[v];
    for (int e = threadIdx.x; e < kGTab; e += blockDim.x) s_tab[e] = P.thr[(size_t)slot * kGTab + e];
    __syncthreads();
    st.bond0 = st.mag0 = st.db = st.dm = 0;
    st.mb = 0;
    st.row = P.row0;
    if (P.bm_known) {
        st.bond0 = P.last_bm[2 * r];
        st.mag0 = P.last_bm[2 * r + 1];
    } else {
        g_measure(P, g_sp, red, st.bond0, st.mag0);
    }
}

// Energy, carried state and spins of replica r at the end of a launch.
__device__ __forceinline__ void graph_finish(const GraphParams& P, int r, const uint8_t* g_sp,
                                             long long bb, long long mm) {
    if (threadIdx.x == 0) {
        P.last_e[r] = -__dmul_rn(P.J, (double)bb);
        P.last_bm[2 * r] = bb;
        P.last_bm[2 * r + 1] = mm;
    }
    uint8_t* spins = P.spins + (size_t)r * P.n;
    for (int v = threadIdx.x; v < P.n; v += blockDim.x) spins[v] = g_sp[v];
}

// n_sweeps sweeps of every replica (block = replica) between exchange points.
__global__ void __launch_bounds__(kGThreads) k_graph_sweeps(const __grid_constant__ GraphParams P) {
    extern __shared__ uint8_t g_sp[];
    __shared__ uint32_t s_tab[kGTab];
    __shared__ int red[64];
    __shared__ long long s_acc[2][2][32];
    const int r = blockIdx.x;
    const int slot = P.r2t[r];
    GState st;
    graph_stage(P, r, slot, g_sp, s_tab, red, st);
    long long bb = 0, mm = 0;
    graph_run(P, r, slot, g_sp, s_tab, s_acc, P.sweep0, P.n_sweeps, P.measure_every,
              P.measure_phase, st, bb, mm);
    graph_finish(P, r, g_sp, bb, mm);
}

// ------------------------------------------------------ persistent PT run
// A whole sampling run in one cooperative launch: between exchange points the
// replicas sweep as above; at an exchange point every block publishes its
// energy, all meet at a grid barrier, and every block computes the same
// exchange pass (the rule of k_graph_exchange) on its own copy of the ladder,
// so the launch needs no second barrier.  Energies alternate between two
// buffers: a block can only rewrite one after every block has passed the
// barrier that follows its reads.  Waits are bounded (kBarrierCycles); a
// timeout sets *err, and every block returns at its next barrier.
__global__ void __launch_bounds__(kGThreads)
    k_graph_pt(const __grid_constant__ GraphParams P, const __grid_constant__ GraphPtParams X) {
    extern __shared__ uint8_t g_sp[];
    __shared__ uint32_t s_tab[kGTab];
    __shared__ int red[64];
    __shared__ long long s_acc[2][2][32];
    __shared__ int s_t2r[kGMaxReplicas];
    __shared__ int s_slot, s_acc_x;
    const int r = blockIdx.x, R = P.R;
    for (int i = threadIdx.x; i < R; i += blockDim.x) s_t2r[i] = X.t2r[i];
    int slot = P.r2t[r];
    GState st;
    graph_stage(P, r, slot, g_sp, s_tab, red, st);
    unsigned long long xc = X.ctrl[0];
    int accepted = 0;
    uint64_t k = X.ksample0;
    int64_t done = 0;
    long long bb = 0, mm = 0;
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    while (done < X.n_sweeps) {
        const uint64_t to_x = (uint64_t)X.ee - (k % (uint64_t)X.ee);
        const int n = (int)min(to_x, (uint64_t)(X.n_sweeps - done));
        const int phase = (int)(((uint64_t)X.me - 1u - (k % (uint64_t)X.me)) % (uint64_t)X.me);
        graph_run(P, r, slot, g_sp, s_tab, s_acc, P.sweep0 + (uint64_t)done, n, X.me, phase, st,
                  bb, mm);
        k += (uint64_t)n;
        done += n;
        if (k % (uint64_t)X.ee != 0) continue;
        // exchange point
        double* eb = X.ebuf + (size_t)(xc & 1ull) * R;
        if (threadIdx.x == 0) {
            eb[r] = -__dmul_rn(P.J, (double)bb);
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
        if (s_slot != slot) {
            slot = s_slot;
            for (int e = threadIdx.x; e < kGTab; e += blockDim.x)
                s_tab[e] = P.thr[(size_t)slot * kGTab + e];
            __syncthreads();
        }
    }
    graph_finish(P, r, g_sp, bb, mm);
    if (threadIdx.x == 0) P.r2t[r] = slot;
    if (r == 0) {
        for (int i = threadIdx.x; i < R; i += blockDim.x) X.t2r[i] = s_t2r[i];
        if (threadIdx.x == 0) {
            X.ctrl[0] = xc;
            X.ctrl[1] += (unsigned long long)accepted;
        }
    }
}

// Hot start of every replica.
__global__ void k_graph_init(uint8_t* spins, int n, int R, uint64_t seed) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t c3 = counter_word3(ISG_TAG_GRAPH, 0xFEu, 0);
    const int64_t total = (int64_t)n * R;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(g / n), v = (int)(g - (int64_t)r * n);
        const U4 u = philox10((uint32_t)r, (uint32_t)v >> 2, 0u, c3, k0, k1);
        const uint32_t jv = (uint32_t)v & 3u;
        const uint32_t w = jv == 0 ? u.x : jv == 1 ? u.y : jv == 2 ? u.z : u.w;
        spins[g] = (uint8_t)(w >> 31);
    }
}

// Exchange pass over the temperature ladder (src/parallel_tempering.rs:16-33)
// on the energies of the replicas' last sweeps, FP64 with explicitly rounded
// products; the parity is the exchange count's.  Shared by the Ising and the
// continuous-spin graph engines.
__global__ void k_graph_exchange(const double* energies, int32_t* r2t, int32_t* t2r,
                                 const double* betas, int R, unsigned long long* ctrl,
                                 uint64_t seed) {
    __shared__ double s_e[kGMaxReplicas];
    __shared__ int s_t2r[kGMaxReplicas];
    __shared__ int s_acc;
    if (threadIdx.x == 0) s_acc = 0;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        s_e[r] = energies[r];
        s_t2r[r] = t2r[r];
    }
    __syncthreads();
    const unsigned long long xc = ctrl[0];
    const int par = (int)(xc & 1ull);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t c3 = counter_word3(ISG_TAG_EXCH, 0, xc);
    for (int i = par + 2 * threadIdx.x; i + 1 < R; i += 2 * blockDim.x) {
        const int ri = s_t2r[i], rj = s_t2r[i + 1];
        const double d = __dmul_rn(__dsub_rn(betas[i], betas[i + 1]), __dsub_rn(s_e[rj], s_e[ri]));
        bool ok = d < 0.0;
        if (!ok) {
            const U4 u = philox10(0xFFFFFFFFu, (uint32_t)i, (uint32_t)xc, c3, k0, k1);
            ok = uniform53(u.x, u.y) < exp(-d);
        }
        if (ok) {
            s_t2r[i] = rj;
            s_t2r[i + 1] = ri;
            r2t[ri] = i + 1;
            r2t[rj] = i;
            atomicAdd(&s_acc, 1);
        }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < R; r += blockDim.x) t2r[r] = s_t2r[r];
    if (threadIdx.x == 0) {
        ctrl[0] = xc + 1;
        ctrl[1] += (unsigned long long)s_acc;
    }
}

// Barrier check: `blocks` co-resident blocks meet at a barrier that expects
// `expected` arrivals, twice.  With expected > blocks nobody releases them, so
// every wait must run out after `limit` cycles and set *err.
__global__ void k_barrier_probe(unsigned int* bar, int* err, unsigned int expected,
                                long long limit) {
    if (!grid_barrier(bar, err, expected, limit)) return;
    grid_barrier(bar, err, expected, limit);
}

cudaError_t launch_graph_exchange(const double* energies, int32_t* r2t, int32_t* t2r,
                                  const double* betas, int R, unsigned long long* ctrl,
                                  uint64_t seed, cudaStream_t stream) {
    k_graph_exchange<<<1, 256, 0, stream>>>(energies, r2t, t2r, betas, R, ctrl, seed);
    return cudaGetLastError();
}

}  // namespace isg

using namespace isg;

struct isg_graph {
    int device = 0;
    int n = 0, m = 0, R = 0, n_classes = 0;
    uint64_t seed = 0;
    double J = 1.0;
    bool temps_set = false;
    uint64_t gsweep = 0;     // global sweep counter
    uint64_t ksample = 0;    // sampling sweeps since reset
    int32_t* d_rowptr = nullptr;
    int32_t* d_adj = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_cstart = nullptr;
    uint8_t* d_spins = nullptr;
    uint32_t* d_thr = nullptr;
    int32_t* d_r2t = nullptr;
    int32_t* d_t2r = nullptr;
    double* d_betas = nullptr;
    double* d_last_e = nullptr;
    long long* d_last_bm = nullptr;
    bool bm_known = false;
    // persistent runs (k_graph_pt): energy buffers, barrier, error flag
    double* d_ebuf = nullptr;
    unsigned int* d_bar = nullptr;
    int* d_err = nullptr;
    bool coop = false;         // all replicas can be resident at once
    unsigned long long* d_ctrl = nullptr;  // [0] exchange count, [1] accepted
    long long* d_rec_b = nullptr;
    long long* d_rec_m = nullptr;
    int32_t* d_rec_t = nullptr;
    int64_t rec_cap = 0;
    cudaStream_t stream = nullptr;
};

namespace {

int g_destroy(isg_graph* H) {
    if (!H) return ISG_OK;
    cudaSetDevice(H->device);
    if (H->stream) cudaStreamSynchronize(H->stream);
    cudaFree(H->d_rowptr);
    cudaFree(H->d_adj);
    cudaFree(H->d_order);
    cudaFree(H->d_cstart);
    cudaFree(H->d_spins);
    cudaFree(H->d_thr);
    cudaFree(H->d_r2t);
    cudaFree(H->d_t2r);
    cudaFree(H->d_betas);
    cudaFree(H->d_last_e);
    cudaFree(H->d_last_bm);
    cudaFree(H->d_ebuf);
    cudaFree(H->d_bar);
    cudaFree(H->d_err);
    cudaFree(H->d_ctrl);
    cudaFree(H->d_rec_b);
    cudaFree(H->d_rec_m);
    cudaFree(H->d_rec_t);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
    return ISG_OK;
}

GraphParams g_params(isg_graph* H) {
    GraphParams P{};
    P.rowptr = H->d_rowptr;
    P.adj = H->d_adj;
    P.order = H->d_order;
    P.cstart = H->d_cstart;
    P.spins = H->d_spins;
    P.thr = H->d_thr;
    P.r2t = H->d_r2t;
    P.rec_b = H->d_rec_b;
    P.rec_m = H->d_rec_m;
    P.rec_t = H->d_rec_t;
    P.last_e = H->d_last_e;
    P.last_bm = H->d_last_bm;
    P.bm_known = H->bm_known ? 1 : 0;
    P.J = H->J;
    P.seed = H->seed;
    P.n = H->n;
    P.R = H->R;
    P.n_classes = H->n_classes;
    return P;
}

int g_launch(isg_graph* H, int n_sweeps, int every, int phase, int64_t row0) {
    GraphParams P = g_params(H);
    P.sweep0 = H->gsweep;
    P.n_sweeps = n_sweeps;
    P.measure_every = every;
    P.measure_phase = phase;
    P.row0 = row0;
    k_graph_sweeps<<<H->R, kGThreads, (size_t)H->n, H->stream>>>(P);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_graph_sweeps");
    H->gsweep += (uint64_t)n_sweeps;
    if (n_sweeps > 0) H->bm_known = true;
    return ISG_OK;
}

}  // namespace

extern "C" {

int isg_graph_create(isg_graph** out, int n_nodes, const int32_t* edges, int n_edges,
                     int replicas, uint64_t seed) {
    if (!out) return fail(ISG_ERR_ARG, "isg_graph_create: out is NULL");
    *out = nullptr;
    if (n_nodes < 1 || n_nodes > kGMaxNodes)
        return fail(ISG_ERR_ARG, "isg_graph_create: n_nodes must be 1..65536");
    if (n_edges < 0 || (n_edges > 0 && !edges))
        return fail(ISG_ERR_ARG, "isg_graph_create: bad edge list");
    if (replicas < 1 || replicas > kGMaxReplicas)
        return fail(ISG_ERR_ARG, "isg_graph_create: replicas must be 1..1024");
    // CSR adjacency (both directions, in edge-list order)
    std::vector<int> deg(n_nodes, 0);
    for (int e = 0; e < n_edges; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || a >= n_nodes || b >= n_nodes)
            return fail(ISG_ERR_ARG, "isg_graph_create: edge " + std::to_string(e) +
                                         " names a node outside 0.." +
                                         std::to_string(n_nodes - 1));
        if (a == b) return fail(ISG_ERR_ARG, "isg_graph_create: self-loop at node " + std::to_string(a));
        ++deg[a];
        ++deg[b];
    }
    for (int v = 0; v < n_nodes; ++v)
        if (deg[v] > kGMaxDeg)
            return fail(ISG_ERR_UNSUPPORTED, "isg_graph_create: node " + std::to_string(v) +
                                                 " has degree " + std::to_string(deg[v]) +
                                                 " (at most 12)");
    std::vector<int32_t> rowptr(n_nodes + 1, 0), adj(2 * (size_t)n_edges);
    for (int v = 0; v < n_nodes; ++v) rowptr[v + 1] = rowptr[v] + deg[v];
    std::vector<int32_t> fillp(rowptr.begin(), rowptr.end() - 1);
    for (int e = 0; e < n_edges; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        adj[fillp[a]++] = b;
        adj[fillp[b]++] = a;
    }
    // greedy proper colouring in node order: smallest class unused by the
    // node's already coloured neighbours
    std::vector<int> col(n_nodes, -1);
    int ncol = 0;
    for (int v = 0; v < n_nodes; ++v) {
        uint32_t used = 0;
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
            if (col[adj[j]] >= 0) used |= 1u << col[adj[j]];
        int c = 0;
        while ((used >> c) & 1u) ++c;
        col[v] = c;
        ncol = std::max(ncol, c + 1);
    }
    std::vector<int32_t> cstart(ncol + 1, 0), order(n_nodes);
    for (int v = 0; v < n_nodes; ++v) ++cstart[col[v] + 1];
    for (int c = 0; c < ncol; ++c) cstart[c + 1] += cstart[c];
    std::vector<int32_t> fillc(cstart.begin(), cstart.end() - 1);
    for (int v = 0; v < n_nodes; ++v) order[fillc[col[v]]++] = v;

    isg_graph* H = new (std::nothrow) isg_graph();
    if (!H) return fail(ISG_ERR_ARG, "isg_graph_create: out of host memory");
    cudaGetDevice(&H->device);
    H->n = n_nodes;
    H->m = n_edges;
    H->R = replicas;
    H->seed = seed;
    H->n_classes = ncol;
    cudaError_t e;
#define GALLOC(ptr, bytes)                                             \
    e = cudaMalloc((void**)&(ptr), std::max<size_t>(4, (bytes)));      \
    if (e != cudaSuccess) {                                            \
        g_destroy(H);                                                  \
        return cuda_fail(e, "cudaMalloc");                             \
    }
    GALLOC(H->d_rowptr, sizeof(int32_t) * (n_nodes + 1));
    GALLOC(H->d_adj, sizeof(int32_t) * adj.size());
    GALLOC(H->d_order, sizeof(int32_t) * n_nodes);
    GALLOC(H->d_cstart, sizeof(int32_t) * (ncol + 1));
    GALLOC(H->d_spins, (size_t)n_nodes * replicas);
    GALLOC(H->d_thr, sizeof(uint32_t) * kGTab * replicas);
    GALLOC(H->d_r2t, sizeof(int32_t) * replicas);
    GALLOC(H->d_t2r, sizeof(int32_t) * replicas);
    GALLOC(H->d_betas, sizeof(double) * replicas);
    GALLOC(H->d_last_e, sizeof(double) * replicas);
    GALLOC(H->d_last_bm, sizeof(long long) * 2 * replicas);
    GALLOC(H->d_ebuf, sizeof(double) * 2 * replicas);
    GALLOC(H->d_bar, sizeof(unsigned int) * 2);
    GALLOC(H->d_err, sizeof(int));
    GALLOC(H->d_ctrl, sizeof(unsigned long long) * 2);
#undef GALLOC
    e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        g_destroy(H);
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    if (n_nodes > 32768) {
        e = cudaFuncSetAttribute(k_graph_sweeps, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 n_nodes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_graph_pt, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     n_nodes);
        if (e != cudaSuccess) {
            g_destroy(H);
            return cuda_fail(e, "cudaFuncSetAttribute");
        }
    }
    {
        // a persistent run needs every replica resident at once
        int coop_attr = 0, sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&coop_attr, cudaDevAttrCooperativeLaunch, H->device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_graph_pt, kGThreads,
                                                          (size_t)n_nodes) != cudaSuccess)
            per_sm = 0;
        cudaGetLastError();
        H->coop = coop_attr && (int64_t)per_sm * sms >= replicas;
    }
    std::vector<int32_t> ident(replicas);
    for (int r = 0; r < replicas; ++r) ident[r] = r;
#define GCK(call)                                                      \
    e = (call);                                                        \
    if (e != cudaSuccess) {                                            \
        g_destroy(H);                                                  \
        return cuda_fail(e, #call);                                    \
    }
    GCK(cudaMemcpyAsync(H->d_rowptr, rowptr.data(), sizeof(int32_t) * rowptr.size(),
                        cudaMemcpyHostToDevice, H->stream));
    if (!adj.empty())
        GCK(cudaMemcpyAsync(H->d_adj, adj.data(), sizeof(int32_t) * adj.size(),
                            cudaMemcpyHostToDevice, H->stream));
    GCK(cudaMemcpyAsync(H->d_order, order.data(), sizeof(int32_t) * n_nodes,
                        cudaMemcpyHostToDevice, H->stream));
    GCK(cudaMemcpyAsync(H->d_cstart, cstart.data(), sizeof(int32_t) * cstart.size(),
                        cudaMemcpyHostToDevice, H->stream));
    GCK(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * replicas,
                        cudaMemcpyHostToDevice, H->stream));
    GCK(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * replicas,
                        cudaMemcpyHostToDevice, H->stream));
    GCK(cudaMemsetAsync(H->d_ctrl, 0, sizeof(unsigned long long) * 2, H->stream));
    GCK(cudaMemsetAsync(H->d_bar, 0, sizeof(unsigned int) * 2, H->stream));
    GCK(cudaMemsetAsync(H->d_err, 0, sizeof(int), H->stream));
    k_graph_init<<<std::max(1, std::min(1024, (n_nodes * replicas + 255) / 256)), 256, 0,
                   H->stream>>>(H->d_spins, n_nodes, replicas, seed);
    GCK(cudaGetLastError());
    GCK(cudaStreamSynchronize(H->stream));
#undef GCK
    *out = H;
    return ISG_OK;
}

int isg_graph_destroy(isg_graph* h) { return g_destroy(h); }

int isg_graph_num_colours(isg_graph* h, int* n) {
    if (!h || !n) return fail(ISG_ERR_ARG, "isg_graph_num_colours: NULL argument");
    *n = h->n_classes;
    return ISG_OK;
}

int isg_graph_set_temperatures(isg_graph* h, const double* temps, double J) {
    if (!h || !temps) return fail(ISG_ERR_ARG, "isg_graph_set_temperatures: NULL argument");
    cudaSetDevice(h->device);
    const int R = h->R;
    std::vector<uint32_t> thr((size_t)kGTab * R, 0u);
    std::vector<double> betas(R);
    for (int t = 0; t < R; ++t) {
        if (!(temps[t] > 0.0) || !std::isfinite(temps[t]))
            return fail(ISG_ERR_ARG, "isg_graph_set_temperatures: temperatures must be positive");
        const double beta = 1.0 / temps[t];
        betas[t] = beta;
        for (int od = 0; od < 2; ++od)
            for (int dg = 0; dg <= kGMaxDeg; ++dg)
                for (int nd = 0; nd <= dg; ++nd) {
                    // dE = 2 J s (sum of neighbours) with s = 1 - 2 od, sum = dg - 2 nd
                    const double dE = 2.0 * J * (od ? -1.0 : 1.0) * (double)(dg - 2 * nd);
                    uint32_t th;
                    if (dE <= 0.0) {
                        th = 0xFFFFFFFFu;
                    } else {
                        double f = std::floor(std::exp(-beta * dE) * 4294967296.0);
                        if (f < 1.0) f = 1.0;
                        th = (uint32_t)(f - 1.0);
                    }
                    thr[(size_t)t * kGTab + (od * (kGMaxDeg + 1) + dg) * (kGMaxDeg + 1) + nd] = th;
                }
    }
    std::vector<int32_t> ident(R);
    for (int r = 0; r < R; ++r) ident[r] = r;
    ISG_CK(cudaMemcpyAsync(h->d_thr, thr.data(), thr.size() * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, h->stream));
    ISG_CK(cudaMemcpyAsync(h->d_betas, betas.data(), sizeof(double) * R, cudaMemcpyHostToDevice,
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

int isg_graph_step(isg_graph* h, int64_t n_sweeps) {
    if (!h) return fail(ISG_ERR_ARG, "isg_graph_step: NULL handle");
    if (!h->temps_set) return fail(ISG_ERR_STATE, "isg_graph_step: temperatures not set");
    if (n_sweeps < 0) return fail(ISG_ERR_ARG, "isg_graph_step: negative sweep count");
    cudaSetDevice(h->device);
    for (int64_t done = 0; done < n_sweeps;) {
        const int n = (int)std::min<int64_t>(n_sweeps - done, 1 << 20);
        int rc = g_launch(h, n, 0, 0, 0);
        if (rc) return rc;
        done += n;
    }
    return ISG_OK;
}

int isg_graph_reset_sampling(isg_graph* h) {
    if (!h) return fail(ISG_ERR_ARG, "isg_graph_reset_sampling: NULL handle");
    cudaSetDevice(h->device);
    ISG_CK(cudaMemsetAsync(h->d_ctrl, 0, sizeof(unsigned long long) * 2, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    h->ksample = 0;
    return ISG_OK;
}

int isg_graph_pt_run(isg_graph* h, int64_t n_sweeps, int exchange_every, int measure_every,
                     int32_t* tslot, int64_t* bond, int64_t* mag, int64_t max_records,
                     int64_t* n_records) {
    if (!h) return fail(ISG_ERR_ARG, "isg_graph_pt_run: NULL handle");
    if (!h->temps_set) return fail(ISG_ERR_STATE, "isg_graph_pt_run: temperatures not set");
    if (n_sweeps < 0 || exchange_every < 1 || measure_every < 1)
        return fail(ISG_ERR_ARG, "isg_graph_pt_run: need n_sweeps >= 0, exchange_every >= 1, "
                                 "measure_every >= 1");
    const uint64_t k0 = h->ksample;
    const int64_t need = (int64_t)((k0 + (uint64_t)n_sweeps) / (uint64_t)measure_every -
                                   k0 / (uint64_t)measure_every);
    if (need > 0 && (!tslot || !bond || !mag || max_records < need))
        return fail(ISG_ERR_ARG, "isg_graph_pt_run: record arrays hold " +
                                     std::to_string(max_records) + " rows, " +
                                     std::to_string(need) + " needed");
    cudaSetDevice(h->device);
    if (need > h->rec_cap) {
        cudaFree(h->d_rec_b);
        cudaFree(h->d_rec_m);
        cudaFree(h->d_rec_t);
        h->d_rec_b = h->d_rec_m = nullptr;
        h->d_rec_t = nullptr;
        h->rec_cap = 0;
        ISG_CK(cudaMalloc((void**)&h->d_rec_b, sizeof(long long) * need * h->R));
        ISG_CK(cudaMalloc((void**)&h->d_rec_m, sizeof(long long) * need * h->R));
        ISG_CK(cudaMalloc((void**)&h->d_rec_t, sizeof(int32_t) * need * h->R));
        h->rec_cap = need;
    }
    int64_t done = 0, row = 0;
    if (h->coop && exchange_every <= 100000 && n_sweeps > 0) {
        // the whole run in one cooperative launch (k_graph_pt)
        GraphParams P = g_params(h);
        P.sweep0 = h->gsweep;
        P.n_sweeps = 0;
        P.measure_every = measure_every;
        P.measure_phase = 0;
        P.row0 = 0;
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
        ISG_CK(cudaLaunchCooperativeKernel((const void*)k_graph_pt, dim3(h->R), dim3(kGThreads),
                                           args, (size_t)h->n, h->stream));
        int err = 0;
        ISG_CK(cudaMemcpyAsync(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        ISG_CK(cudaStreamSynchronize(h->stream));
        if (err)
            return fail(ISG_ERR_TIMEOUT, "isg_graph_pt_run: a replica did not reach the exchange "
                                         "barrier in time");
        h->gsweep += (uint64_t)n_sweeps;
        h->ksample += (uint64_t)n_sweeps;
        h->bm_known = true;
        done = n_sweeps;
        row = need;
    }
    // runs of sweeps between exchange points; each ends with the exchange pass
    while (done < n_sweeps) {
        const uint64_t k = h->ksample;
        const uint64_t to_x = (uint64_t)exchange_every - (k % (uint64_t)exchange_every);
        const int n = (int)std::min<uint64_t>(to_x, (uint64_t)(n_sweeps - done));
        // measured sweeps of this run: local j with (k + j + 1) % measure_every == 0
        const int phase = (int)(((uint64_t)measure_every - 1u - (k % (uint64_t)measure_every)) %
                                (uint64_t)measure_every);
        int rc = g_launch(h, n, measure_every, phase, row);
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
        ISG_CK(cudaMemcpyAsync(bond, h->d_rec_b, sizeof(long long) * row * h->R,
                               cudaMemcpyDeviceToHost, h->stream));
        ISG_CK(cudaMemcpyAsync(mag, h->d_rec_m, sizeof(long long) * row * h->R,
                               cudaMemcpyDeviceToHost, h->stream));
    }
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

int isg_graph_get_accepted(isg_graph* h, int64_t* accepted) {
    if (!h || !accepted) return fail(ISG_ERR_ARG, "isg_graph_get_accepted: NULL argument");
    cudaSetDevice(h->device);
    unsigned long long c[2];
    ISG_CK(cudaMemcpyAsync(c, h->d_ctrl, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    *accepted = (int64_t)c[1];
    return ISG_OK;
}

int isg_graph_get_spins(isg_graph* h, int replica, int8_t* out) {
    if (!h || !out || replica < 0 || replica >= h->R)
        return fail(ISG_ERR_ARG, "isg_graph_get_spins: bad argument");
    cudaSetDevice(h->device);
    std::vector<uint8_t> d(h->n);
    ISG_CK(cudaMemcpyAsync(d.data(), h->d_spins + (size_t)replica * h->n, h->n,
                           cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    for (int v = 0; v < h->n; ++v) out[v] = d[v] ? (int8_t)-1 : (int8_t)1;
    return ISG_OK;
}

int isg_barrier_selftest(int blocks, int expected, int64_t limit_cycles, int* timed_out) {
    if (blocks < 1 || expected < 1 || limit_cycles < 1 || !timed_out)
        return fail(ISG_ERR_ARG, "isg_barrier_selftest: bad argument");
    int dev = 0, sms = 0, coop = 0;
    ISG_CK(cudaGetDevice(&dev));
    ISG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ISG_CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return fail(ISG_ERR_UNSUPPORTED, "isg_barrier_selftest: no cooperative launch");
    if (blocks > sms) return fail(ISG_ERR_ARG, "isg_barrier_selftest: blocks must fit one per SM");
    unsigned int* bar = nullptr;
    int* err = nullptr;
    ISG_CK(cudaMalloc((void**)&bar, sizeof(unsigned int) * 2));
    cudaError_t e = cudaMalloc((void**)&err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(bar, 0, sizeof(unsigned int) * 2);
    if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
    unsigned int ex = (unsigned int)expected;
    long long lim = (long long)limit_cycles;
    void* args[] = {&bar, &err, &ex, &lim};
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(blocks), dim3(64), args,
                                        0, nullptr);
    int host_err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&host_err, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(err);
    if (e != cudaSuccess) return cuda_fail(e, "isg_barrier_selftest");
    *timed_out = host_err;
    return ISG_OK;
}

int isg_graph_get_r2t(isg_graph* h, int32_t* r2t) {
    if (!h || !r2t) return fail(ISG_ERR_ARG, "isg_graph_get_r2t: NULL argument");
    cudaSetDevice(h->device);
    ISG_CK(cudaMemcpyAsync(r2t, h->d_r2t, sizeof(int32_t) * h->R, cudaMemcpyDeviceToHost,
                           h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

}  // extern "C"
