// isg_cont.cu — continuous-spin O(n) models (n = 3 Heisenberg, n = 2 XY) on
// periodic cubic lattices: checkerboard Metropolis with a cone proposal,
// microcanonical overrelaxation, deterministic observables summed exactly in
// fixed point (2^-24) and converted to FP64 at the combine, device replica
// exchange and the PT cycle as a graph.
//
// Reference path being replaced (faulknco/ising-rs):
//   src/cuda/continuous_spin_kernel.cu:9-142  Metropolis + overrelaxation
//   src/cuda/reduce_kernel.cu:70-151          vector M and energy partials
//   src/cuda/gpu_lattice_continuous.rs:24-240 ContinuousGpuLattice
//   src/bin/gpu_fss.rs:414-582                run_continuous_fss
// Proposal: a uniform rotation inside a cone of half-angle delta around the
// current spin (the reference CPU proposal, heisenberg/metropolis.rs:54-92;
// the reference GPU kernel perturbs in a box and renormalises,
// continuous_spin_kernel.cu:58-71).  XY: angle step uniform in
// [-delta, delta] (delta >= pi gives a uniform new angle).
//
// Layout in HBM: per (size, replica) lattice, FP32 component planes split by
// colour: [colour][component][L^3/2] floats, colour index (z*L*L+y*L+x) >> 1,
// so a warp reads 128 contiguous bytes per component.  XY spins are stored as
// (cos, sin) pairs (8 B/site): every neighbour field is then a plain sum, with
// no trigonometry per neighbour.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {

constexpr int kCMaxClasses = 16;
constexpr int kCMaxReplicas = 1024;
constexpr int kCThreads = 256;
constexpr int kNQ = 10;              // E, Mx, My, Mz, Cx, Cy, Cz, Sx, Sy, Sz

struct ContClass {
    int L;
    int R;
    uint32_t plane_sites;
    FastDiv div_half;   // L/2
    FastDiv div_L;
    FastDiv div_plane;  // plane_sites (used when R * plane_sites < 2^31)
    int small;
    int rep_base;
    int64_t off;        // float offset of replica 0
    int64_t site_base;  // flattened colour-plane sites
    int64_t site_end;
    int chunk_base;
    int chunks_per_rep;
    int nseg;           // z segments of kColZ planes per column
    int64_t col_base;   // column tasks (replica, z segment, colour index in a z-plane)
    int64_t col_end;
};

// Column tasks of the half-sweep kernels: a thread updates the sites of one
// colour at colour index col of z-planes [zseg*kColZ, min(L, (zseg+1)*kColZ))
// of one replica, walking z; a warp covers 32 consecutive col values.
constexpr int kColZ = 32;

struct ContParams {
    float* spins;
    const float* betaf;  // per slot
    const int32_t* r2t;
    unsigned long long* ctrl;  // [0] sweep base
    unsigned long long* metro_acc;
    long long* partials;       // [chunks][kNQ] fixed-point block sums (2^-24 units)
    uint32_t rk0[10], rk1[10]; // Philox round keys of the seed
    uint64_t seed;
    float J;
    double Jd;
    int n_classes;
    int renorm;
    int64_t total_sites;
    int64_t total_cols;
    int total_chunks;
    ContClass cls[kCMaxClasses];
};

template <int NC>
__device__ __forceinline__ int64_t plane_off(const ContClass& C, int r, int colour, int comp) {
    return C.off + (int64_t)r * 2 * NC * C.plane_sites +
           (int64_t)(colour * NC + comp) * C.plane_sites;
}

// Position of a column task.
struct ColRef {
    int ci, r, rg;
    uint32_t col, y, k, z0, z1, Pz;
};
__device__ __forceinline__ bool col_locate(const ContParams& P, int64_t t, ColRef& c) {
    if (t >= P.total_cols) return false;
    int ci = 0;
    while (P.cls[ci].col_end <= t) ++ci;
    const ContClass& C = P.cls[ci];
    const uint32_t L = (uint32_t)C.L, half = L >> 1;
    c.ci = ci;
    c.Pz = L * half;  // colour sites per z-plane
    const int64_t tl = t - C.col_base;
    const int64_t rem = tl / c.Pz;
    c.col = (uint32_t)(tl - rem * c.Pz);
    const int zseg = (int)(rem % C.nseg);
    c.r = (int)(rem / C.nseg);
    c.rg = C.rep_base + c.r;
    c.y = fdiv(c.col, C.div_half);
    c.k = c.col - c.y * half;
    c.z0 = (uint32_t)zseg * kColZ;
    c.z1 = min(L, c.z0 + (uint32_t)kColZ);
    return true;
}

// Neighbour field of the site at (colour index col, plane z) of colour
// `colour`, summed in the order x+, x-, y+, y-, z+, z- as
// ((x+ + x-) + (y+ + y-)) + (z+ + z-).  zc = other colour at (z, col) (one of
// the two x-neighbours), zm = at (z-1, col); returns z+ = at (z+1, col) in zp.
template <int NC>
__device__ __forceinline__ void col_field(const float* oth, uint32_t plane, uint32_t zb,
                                          uint32_t zpb, uint32_t col, uint32_t xo, uint32_t colp,
                                          uint32_t colm, uint32_t p, const float (&zc)[NC],
                                          const float (&zm)[NC], float (&zp)[NC], float (&h)[NC]) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        const float* o = oth + (size_t)k * plane;
        const float xn = __ldg(o + zb + xo);
        const float yp = __ldg(o + zb + colp);
        const float ym = __ldg(o + zb + colm);
        zp[k] = __ldg(o + zpb + col);
        const float xp = p ? xn : zc[k], xm = p ? zc[k] : xn;
        h[k] = ((xp + xm) + (yp + ym)) + (zp[k] + zm[k]);
    }
}

// Overrelaxation half-sweep on column tasks: S' = 2 (S.h)/|h|^2 h - S about the
// local field (continuous_spin_kernel.cu:88-142; overrelax.rs:16-49 without the
// per-update renormalisation), skipped where |h|^2 < 1e-20.  The
// next z-step's loads are issued before the current step's arithmetic.
template <int NC>
__global__ void __launch_bounds__(kCThreads) k_cont_or_col(const __grid_constant__ ContParams P,
                                                           int colour) {
    ColRef c;
    if (!col_locate(P, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, c)) return;
    const ContClass& C = P.cls[c.ci];
    const uint32_t L = (uint32_t)C.L, half = L >> 1, plane = C.plane_sites;
    float* own = P.spins + plane_off<NC>(C, c.r, colour, 0);
    const float* oth = P.spins + plane_off<NC>(C, c.r, colour ^ 1, 0);
    const uint32_t row = c.y * half;
    const uint32_t xo1 = row + (c.k + 1 == half ? 0 : c.k + 1);  // x+ when the site is odd
    const uint32_t xo0 = row + (c.k == 0 ? half - 1 : c.k - 1);  // x- when the site is even
    const uint32_t colp = (c.y + 1 == L ? 0 : c.y + 1) * half + c.k;
    const uint32_t colm = (c.y == 0 ? L - 1 : c.y - 1) * half + c.k;
    float zm[NC], zc[NC];
    const uint32_t zmb = (c.z0 == 0 ? L - 1 : c.z0 - 1) * c.Pz;
    // loads of step z: x-neighbour (not at col), y+, y-, z+ (other colour), own
    float lx[NC], lyp[NC], lym[NC], lzp[NC], lv[NC];
    auto load_step = [&](uint32_t z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz, zpb = (z + 1 == L ? 0 : z + 1) * c.Pz;
        const uint32_t xo = p ? xo1 : xo0;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float* o = oth + (size_t)k * plane;
            lx[k] = __ldg(o + zb + xo);
            lyp[k] = __ldg(o + zb + colp);
            lym[k] = __ldg(o + zb + colm);
            lzp[k] = __ldg(o + zpb + c.col);
            lv[k] = own[(size_t)k * plane + zb + c.col];
        }
    };
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        zm[k] = __ldg(oth + (size_t)k * plane + zmb + c.col);
        zc[k] = __ldg(oth + (size_t)k * plane + c.z0 * c.Pz + c.col);
    }
    load_step(c.z0);
    for (uint32_t z = c.z0; z < c.z1; ++z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz;
        float xn[NC], yp[NC], ym[NC], zp[NC], v[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            xn[k] = lx[k];
            yp[k] = lyp[k];
            ym[k] = lym[k];
            zp[k] = lzp[k];
            v[k] = lv[k];
        }
        if (z + 1 < c.z1) load_step(z + 1);
        float h[NC], h2 = 0.f, sh = 0.f;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float xp = p ? xn[k] : zc[k], xm = p ? zc[k] : xn[k];
            h[k] = ((xp + xm) + (yp[k] + ym[k])) + (zp[k] + zm[k]);
            h2 = fmaf(h[k], h[k], h2);
            sh = fmaf(v[k], h[k], sh);
        }
        if (h2 >= 1e-20f) {
            const float scale = 2.0f * sh / h2;
#pragma unroll
            for (int k = 0; k < NC; ++k) own[(size_t)k * plane + zb + c.col] = fmaf(scale, h[k], -v[k]);
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            zm[k] = zc[k];
            zc[k] = zp[k];
        }
    }
}

// Overrelaxation on column tasks of two adjacent sites (colour indices k, k+1
// of one row; every size a multiple of 4, so rows hold an even number of
// colour sites): pair task t is column task 2t.  Own, y+, y-, z+ words are
// 64-bit loads of the pair; of the x neighbours, one per site is the other
// site's same-index word (zc) and one scalar load per pair brings the outer
// one.  Each site's arithmetic is k_cont_or_col's, in the same order; a site
// whose field vanishes is written back unchanged.
template <int NC>
__global__ void __launch_bounds__(kCThreads, 3) k_cont_or_col2(const __grid_constant__ ContParams P,
                                                            int colour) {
    ColRef c;
    if (!col_locate(P, 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x), c)) return;
    const ContClass& C = P.cls[c.ci];
    const uint32_t L = (uint32_t)C.L, half = L >> 1, plane = C.plane_sites;
    float* own = P.spins + plane_off<NC>(C, c.r, colour, 0);
    const float* oth = P.spins + plane_off<NC>(C, c.r, colour ^ 1, 0);
    const uint32_t row = c.y * half;
    const uint32_t xo1 = row + (c.k + 2 == half ? 0 : c.k + 2);  // x+ of site k+1 (p = 1)
    const uint32_t xo0 = row + (c.k == 0 ? half - 1 : c.k - 1);  // x- of site k (p = 0)
    const uint32_t colp = (c.y + 1 == L ? 0 : c.y + 1) * half + c.k;
    const uint32_t colm = (c.y == 0 ? L - 1 : c.y - 1) * half + c.k;
    float2 zm[NC], zc[NC];
    const uint32_t zmb = (c.z0 == 0 ? L - 1 : c.z0 - 1) * c.Pz;
    float lx[NC];
    float2 lyp[NC], lym[NC], lzp[NC], lv[NC];
    auto ld2 = [](const float* q) { return __ldg(reinterpret_cast<const float2*>(q)); };
    auto load_step = [&](uint32_t z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz, zpb = (z + 1 == L ? 0 : z + 1) * c.Pz;
        const uint32_t xo = p ? xo1 : xo0;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float* o = oth + (size_t)k * plane;
            lx[k] = __ldg(o + zb + xo);
            lyp[k] = ld2(o + zb + colp);
            lym[k] = ld2(o + zb + colm);
            lzp[k] = ld2(o + zpb + c.col);
            lv[k] = *reinterpret_cast<const float2*>(own + (size_t)k * plane + zb + c.col);
        }
    };
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        zm[k] = ld2(oth + (size_t)k * plane + zmb + c.col);
        zc[k] = ld2(oth + (size_t)k * plane + c.z0 * c.Pz + c.col);
    }
    load_step(c.z0);
    for (uint32_t z = c.z0; z < c.z1; ++z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz;
        float xn[NC];
        float2 yp[NC], ym[NC], zp[NC], v[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            xn[k] = lx[k];
            yp[k] = lyp[k];
            ym[k] = lym[k];
            zp[k] = lzp[k];
            v[k] = lv[k];
        }
        if (z + 1 < c.z1) load_step(z + 1);
        float ha[NC], hb[NC], h2a = 0.f, sha = 0.f, h2b = 0.f, shb = 0.f;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            // site k: x neighbours (zc.y, zc.x) for p = 1, (zc.x, xn) for p = 0
            const float xpa = p ? zc[k].y : zc[k].x, xma = p ? zc[k].x : xn[k];
            // site k+1: (xn, zc.y) for p = 1, (zc.y, zc.x) for p = 0
            const float xpb = p ? xn[k] : zc[k].y, xmb = p ? zc[k].y : zc[k].x;
            ha[k] = ((xpa + xma) + (yp[k].x + ym[k].x)) + (zp[k].x + zm[k].x);
            hb[k] = ((xpb + xmb) + (yp[k].y + ym[k].y)) + (zp[k].y + zm[k].y);
            h2a = fmaf(ha[k], ha[k], h2a);
            sha = fmaf(v[k].x, ha[k], sha);
            h2b = fmaf(hb[k], hb[k], h2b);
            shb = fmaf(v[k].y, hb[k], shb);
        }
        const bool ua = h2a >= 1e-20f, ub = h2b >= 1e-20f;
        if (ua || ub) {
            const float sca = ua ? 2.0f * sha / h2a : 0.f, scb = ub ? 2.0f * shb / h2b : 0.f;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                float2 w;
                w.x = ua ? fmaf(sca, ha[k], -v[k].x) : v[k].x;
                w.y = ub ? fmaf(scb, hb[k], -v[k].y) : v[k].y;
                *reinterpret_cast<float2*>(own + (size_t)k * plane + zb + c.col) = w;
            }
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            zm[k] = zc[k];
            zc[k] = zp[k];
        }
    }
}

// k_cont_or_col2 with the loads of a step through a per-thread ring of kOrStages stages in
// shared memory (cp.async, two steps ahead), laid out item by item over the
// block's threads so that a warp's reads are conflict-free: per stage and
// component the outer x word (4 B), then the y+, y-, z+ and own pairs (8 B).
// Only the issuing thread reads its copies, so no barrier is needed.
constexpr int kOrStages = 3;
constexpr uint32_t kOrCompBytes = (uint32_t)kCThreads * (4 + 4 * 8);
template <int NC>
constexpr size_t or_ring_bytes() { return (size_t)kOrStages * NC * kOrCompBytes; }

__device__ __forceinline__ void cp_async_ca4(uint32_t saddr, const void* g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_ca8(uint32_t saddr, const void* g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ float lds_f32(uint32_t saddr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(saddr) : "memory");
    return v;
}
__device__ __forceinline__ float2 lds_f2(uint32_t saddr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(saddr) : "memory");
    return v;
}

// Used for O(2): 3 blocks per SM fit their rings and the loads run two steps
// ahead (5% faster than k_cont_or_col2); O(3)'s larger rings allow 2 blocks
// per SM, and there the register form is faster.
template <int NC>
__global__ void __launch_bounds__(kCThreads, 3) k_cont_or_ring2(const __grid_constant__ ContParams P,
                                                             int colour) {
    extern __shared__ __align__(16) unsigned char s_or[];
    ColRef c;
    if (!col_locate(P, 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x), c)) return;
    const ContClass& C = P.cls[c.ci];
    const uint32_t L = (uint32_t)C.L, half = L >> 1, plane = C.plane_sites;
    float* own = P.spins + plane_off<NC>(C, c.r, colour, 0);
    const float* oth = P.spins + plane_off<NC>(C, c.r, colour ^ 1, 0);
    const uint32_t row = c.y * half;
    const uint32_t xo1 = row + (c.k + 2 == half ? 0 : c.k + 2);  // x+ of site k+1 (p = 1)
    const uint32_t xo0 = row + (c.k == 0 ? half - 1 : c.k - 1);  // x- of site k (p = 0)
    const uint32_t colp = (c.y + 1 == L ? 0 : c.y + 1) * half + c.k;
    const uint32_t colm = (c.y == 0 ? L - 1 : c.y - 1) * half + c.k;
    const uint32_t tb = (uint32_t)__cvta_generic_to_shared(s_or) + threadIdx.x * 4u;
    // copies of step z into stage st: per component the outer x word, the
    // y+, y-, z+ and own pairs; one commit group per step
    auto issue = [&](uint32_t z, uint32_t st) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz, zpb = (z + 1 == L ? 0 : z + 1) * c.Pz;
        const uint32_t xo = p ? xo1 : xo0;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float* o = oth + (size_t)k * plane;
            const uint32_t cb = tb + (st * NC + (uint32_t)k) * kOrCompBytes;
            const uint32_t c8 = cb + threadIdx.x * 4u + kCThreads * 4u;  // pair items
            cp_async_ca4(cb, o + zb + xo);
            cp_async_ca8(c8, o + zb + colp);
            cp_async_ca8(c8 + kCThreads * 8u, o + zb + colm);
            cp_async_ca8(c8 + kCThreads * 16u, o + zpb + c.col);
            cp_async_ca8(c8 + kCThreads * 24u, own + (size_t)k * plane + zb + c.col);
        }
        cp_async_commit();
    };
    float2 zm[NC], zc[NC];
    const uint32_t zmb = (c.z0 == 0 ? L - 1 : c.z0 - 1) * c.Pz;
    auto ld2 = [](const float* q) { return __ldg(reinterpret_cast<const float2*>(q)); };
    issue(c.z0, 0);
    if (c.z0 + 1 < c.z1) issue(c.z0 + 1, 1);
    else cp_async_commit();
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        zm[k] = ld2(oth + (size_t)k * plane + zmb + c.col);
        zc[k] = ld2(oth + (size_t)k * plane + c.z0 * c.Pz + c.col);
    }
    uint32_t st = 0;  // stage of step z
    for (uint32_t z = c.z0; z < c.z1; ++z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz;
        // step z + 2 into the stage step z - 1 used (this thread read it)
        if (z + 2 < c.z1) issue(z + 2, st == 0 ? 2u : st - 1);
        else cp_async_commit();
        cp_async_wait<2>();
        float xn[NC];
        float2 yp[NC], ym[NC], zp[NC], v[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const uint32_t cb = tb + (st * NC + (uint32_t)k) * kOrCompBytes;
            const uint32_t c8 = cb + threadIdx.x * 4u + kCThreads * 4u;
            xn[k] = lds_f32(cb);
            yp[k] = lds_f2(c8);
            ym[k] = lds_f2(c8 + kCThreads * 8u);
            zp[k] = lds_f2(c8 + kCThreads * 16u);
            v[k] = lds_f2(c8 + kCThreads * 24u);
        }
        st = st == 2 ? 0u : st + 1;
        float ha[NC], hb[NC], h2a = 0.f, sha = 0.f, h2b = 0.f, shb = 0.f;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            // site k: x neighbours (zc.y, zc.x) for p = 1, (zc.x, xn) for p = 0
            const float xpa = p ? zc[k].y : zc[k].x, xma = p ? zc[k].x : xn[k];
            // site k+1: (xn, zc.y) for p = 1, (zc.y, zc.x) for p = 0
            const float xpb = p ? xn[k] : zc[k].y, xmb = p ? zc[k].y : zc[k].x;
            ha[k] = ((xpa + xma) + (yp[k].x + ym[k].x)) + (zp[k].x + zm[k].x);
            hb[k] = ((xpb + xmb) + (yp[k].y + ym[k].y)) + (zp[k].y + zm[k].y);
            h2a = fmaf(ha[k], ha[k], h2a);
            sha = fmaf(v[k].x, ha[k], sha);
            h2b = fmaf(hb[k], hb[k], h2b);
            shb = fmaf(v[k].y, hb[k], shb);
        }
        const bool ua = h2a >= 1e-20f, ub = h2b >= 1e-20f;
        if (ua || ub) {
            const float sca = ua ? 2.0f * sha / h2a : 0.f, scb = ub ? 2.0f * shb / h2b : 0.f;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                float2 w;
                w.x = ua ? fmaf(sca, ha[k], -v[k].x) : v[k].x;
                w.y = ub ? fmaf(scb, hb[k], -v[k].y) : v[k].y;
                *reinterpret_cast<float2*>(own + (size_t)k * plane + zb + c.col) = w;
            }
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            zm[k] = zc[k];
            zc[k] = zp[k];
        }
    }
}

// The Metropolis move of one site (k_cont_metro_col and its two-site form):
// the cone proposal w of spin v from Philox block u (O(3): polar angle with
// cos uniform in [cos delta, 1], azimuth uniform, about v; O(2): rotation by
// an angle uniform in [-delta, delta]), and the test against field h.
template <int NC>
__device__ __forceinline__ bool cone_test(const float (&v)[NC], const float (&h)[NC], const U4& u,
                                          float cos_delta, float delta, float beta, float J,
                                          float (&w)[NC]) {
    if constexpr (NC == 3) {
        const float ct = 1.0f - uniform24(u.x) * (1.0f - cos_delta);
        const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        // azimuth 2 pi u1: sin and cos of 2 pi u1 - pi (inside [-pi, pi),
        // where the fast intrinsics are accurate to a few 1e-7), negated
        float sp, cp;
        __sincosf(6.28318530717958648f * uniform24(u.y) - 3.14159265358979324f, &sp, &cp);
        sp = -sp;
        cp = -cp;
        const float tx = fabsf(v[0]) < 0.9f ? 1.0f : 0.0f;
        const float ty = 1.0f - tx;
        const float ts = tx * v[0] + ty * v[1];
        float ux = tx - ts * v[0], uy = ty - ts * v[1], uz = -ts * v[2];
        const float un = rsqrtf(ux * ux + uy * uy + uz * uz);
        ux *= un;
        uy *= un;
        uz *= un;
        const float vx = v[1] * uz - v[2] * uy;
        const float vy = v[2] * ux - v[0] * uz;
        const float vz = v[0] * uy - v[1] * ux;
        const float a = st * cp, b = st * sp;
        w[0] = a * ux + b * vx + ct * v[0];
        w[1] = a * uy + b * vy + ct * v[1];
        w[2] = a * uz + b * vz + ct * v[2];
        const float wn = rsqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) w[k] *= wn;
    } else {
        float sd, cd;  // angle in [-delta, delta], delta <= pi
        __sincosf(delta * (2.0f * uniform24(u.x) - 1.0f), &sd, &cd);
        w[0] = v[0] * cd - v[1] * sd;
        w[1] = v[1] * cd + v[0] * sd;
    }
    float dot = 0.f;
#pragma unroll
    for (int k = 0; k < NC; ++k) dot = fmaf(w[k] - v[k], h[k], dot);
    const float dE = -J * dot;
    return dE <= 0.0f || uniform24(u.z) < __expf(-beta * dE);
}

// Metropolis with the cone proposal on column tasks (continuous_spin_kernel.cu:9-83
// with the cone proposal of heisenberg/metropolis.rs:54-69): O(3) one Philox block
// per site at its colour index i (words x, y, z); O(2) one block per colour-index
// pair at i >> 1 (words x, z for even i, y, w for odd i); on renormalisation
// sweeps every site of this colour is written back normalised.
template <int NC>
__global__ void __launch_bounds__(kCThreads, 3)
    k_cont_metro_col(const __grid_constant__ ContParams P, int colour, int sweep_off,
                     float cos_delta, float delta) {
    const uint64_t sweep = P.ctrl[0] + (uint64_t)sweep_off;
    const bool renorm_now = P.renorm > 0 && ((sweep + 1) % (uint64_t)P.renorm) == 0;
    const uint32_t c2 = (uint32_t)sweep;
    const uint32_t c3 = counter_word3(ISG_TAG_CMETRO, (uint32_t)colour, sweep);
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const int lane = threadIdx.x & 31;
    ColRef c;
    const bool live = col_locate(P, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, c);
    unsigned n_acc = 0;
    int rg = -1;
    if (live) {
        const ContClass& C = P.cls[c.ci];
        rg = c.rg;
        const uint32_t L = (uint32_t)C.L, half = L >> 1, plane = C.plane_sites;
        float* own = P.spins + plane_off<NC>(C, c.r, colour, 0);
        const float* oth = P.spins + plane_off<NC>(C, c.r, colour ^ 1, 0);
        const uint32_t row = c.y * half;
        const uint32_t xo1 = row + (c.k + 1 == half ? 0 : c.k + 1);
        const uint32_t xo0 = row + (c.k == 0 ? half - 1 : c.k - 1);
        const uint32_t colp = (c.y + 1 == L ? 0 : c.y + 1) * half + c.k;
        const uint32_t colm = (c.y == 0 ? L - 1 : c.y - 1) * half + c.k;
        const uint32_t uid = replica_uid(C.L, c.r);
        // the warp-uniform part of the Philox rounds (counter {uid, i, c2, c3})
        const PhiloxPre pre = philox_pre(uid, c2, c3, k0, k1);
        const float beta = P.betaf[C.rep_base + P.r2t[c.rg]];
        float zm[NC], zc[NC];
        const uint32_t zmb = (c.z0 == 0 ? L - 1 : c.z0 - 1) * c.Pz;
        // loads of step z, issued one step ahead
        float lx[NC], lyp[NC], lym[NC], lzp[NC], lv[NC];
        auto load_step = [&](uint32_t z) {
            const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
            const uint32_t zb = z * c.Pz, zpb = (z + 1 == L ? 0 : z + 1) * c.Pz;
            const uint32_t xo = p ? xo1 : xo0;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const float* o = oth + (size_t)k * plane;
                lx[k] = __ldg(o + zb + xo);
                lyp[k] = __ldg(o + zb + colp);
                lym[k] = __ldg(o + zb + colm);
                lzp[k] = __ldg(o + zpb + c.col);
                lv[k] = own[(size_t)k * plane + zb + c.col];
            }
        };
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            zm[k] = __ldg(oth + (size_t)k * plane + zmb + c.col);
            zc[k] = __ldg(oth + (size_t)k * plane + c.z0 * c.Pz + c.col);
        }
        load_step(c.z0);
        for (uint32_t z = c.z0; z < c.z1; ++z) {
            const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
            const uint32_t zb = z * c.Pz;
            const uint32_t i = zb + c.col;
            float h[NC], zp[NC], v[NC], w[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const float xn = lx[k];
                const float xp = p ? xn : zc[k], xm = p ? zc[k] : xn;
                zp[k] = lzp[k];
                h[k] = ((xp + xm) + (lyp[k] + lym[k])) + (zp[k] + zm[k]);
                v[k] = lv[k];
            }
            if (z + 1 < c.z1) load_step(z + 1);
            // O(3): one block per site; O(2): one block per colour-index pair,
            // words (x, z) for the even index, (y, w) for the odd
            U4 u = philox_w(pre, P, NC == 3 ? i : i >> 1);
            if (NC == 2 && (i & 1u)) u = U4{u.y, u.x, u.w, u.z};
            const bool accepted = cone_test<NC>(v, h, u, cos_delta, delta, beta, P.J, w);
            n_acc += accepted ? 1u : 0u;
            if (accepted || renorm_now) {
                float n2 = 0.f;
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    if (accepted) v[k] = w[k];
                    n2 = fmaf(v[k], v[k], n2);
                }
                const float sc = renorm_now ? rsqrtf(n2) : 1.0f;
#pragma unroll
                for (int k = 0; k < NC; ++k) own[(size_t)k * plane + i] = v[k] * sc;
            }
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                zm[k] = zc[k];
                zc[k] = zp[k];
            }
        }
    }
    // per-replica acceptance count: a warp covers one replica (32 | colour
    // sites per z-plane), so one atomic per warp
    const int rg0 = __shfl_sync(ISG_FULL_MASK, rg, 0);
    const unsigned cnt = __reduce_add_sync(ISG_FULL_MASK, n_acc);
    if (__all_sync(ISG_FULL_MASK, rg == rg0 || rg < 0)) {
        if (lane == 0 && rg0 >= 0 && cnt) atomicAdd(&P.metro_acc[rg0], (unsigned long long)cnt);
    } else if (rg >= 0 && n_acc) {
        atomicAdd(&P.metro_acc[rg], (unsigned long long)n_acc);
    }
}

// Fixed-point sums of the measurement: every term (a spin component, a bond
// product S.S' or (S x S')_z, all of magnitude <= 1 up to FP32 drift) is
// rounded once to a multiple of 2^-24 and summed exactly in integers: int32
// per thread (at most 32 terms of 2^24: < 2^30), int64 across threads and
// blocks.  Exact integer sums do not depend on the order of summation; the
// only rounding is the one per term, below the FP32 rounding of the products.
constexpr float kFix = 16777216.0f;  // 2^24
__device__ __forceinline__ int fx(float x) { return __float2int_rn(x * kFix); }

// The six bonds of one colour-1 site s with neighbours n (x+, x-, y+, y-,
// z+, z-) into the sums: per axis a the forward bond (i, i+a) and the
// backward bond (i-a, i), C_a += S.S, S_a += (S x S')_z.  E = -J (C_x + C_y +
// C_z) is formed at the combine.
template <int NC>
__device__ __forceinline__ void meas_bonds(int (&acc)[kNQ], const float (&s)[NC],
                                           const float (&n)[6][NC]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float cf = 0.f, cb = 0.f;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            cf = fmaf(s[c], n[2 * a][c], cf);
            cb = fmaf(s[c], n[2 * a + 1][c], cb);
        }
        const float sf = s[0] * n[2 * a][1] - s[1] * n[2 * a][0];
        const float sb = n[2 * a + 1][0] * s[1] - n[2 * a + 1][1] * s[0];
        acc[4 + a] += fx(cf) + fx(cb);
        acc[7 + a] += fx(sf) + fx(sb);
    }
}

__device__ __forceinline__ void meas_block_store(const ContParams& P, int (&acc)[kNQ], int chunk);

// Metropolis on column tasks of two adjacent sites (the pair layout of
// k_cont_or_col2): each site draws the Philox words k_cont_metro_col gives it
// (O(3): its own block; O(2): the pair's one block) and goes through cone_test
// exactly as there; a site neither accepted nor renormalised is written back
// unchanged.  With MEAS (the last half-sweep of a measured sweep, colour 1),
// each pair's final spins and their six neighbours of colour 0 (final too)
// also go into the fixed-point sums, in the order and with the thread layout
// of k_cont_measure2, so the fused sums equal a separate measurement bit for
// bit.
template <int NC, bool MEAS>
__device__ __forceinline__ void metro2_column(const ContParams& P, const ColRef& c, int colour,
                                              uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                              float cos_delta, float delta, bool renorm_now,
                                              unsigned& n_acc, int (&acc)[kNQ]) {
    const ContClass& C = P.cls[c.ci];
    const uint32_t L = (uint32_t)C.L, half = L >> 1, plane = C.plane_sites;
    float* own = P.spins + plane_off<NC>(C, c.r, colour, 0);
    const float* oth = P.spins + plane_off<NC>(C, c.r, colour ^ 1, 0);
    const uint32_t row = c.y * half;
    const uint32_t xo1 = row + (c.k + 2 == half ? 0 : c.k + 2);  // x+ of site k+1 (p = 1)
    const uint32_t xo0 = row + (c.k == 0 ? half - 1 : c.k - 1);  // x- of site k (p = 0)
    const uint32_t colp = (c.y + 1 == L ? 0 : c.y + 1) * half + c.k;
    const uint32_t colm = (c.y == 0 ? L - 1 : c.y - 1) * half + c.k;
    const uint32_t uid = replica_uid(C.L, c.r);
    // the warp-uniform part of the Philox rounds (counter {uid, i, c2, c3})
    const PhiloxPre pre = philox_pre(uid, c2, c3, k0, k1);
    const float beta = P.betaf[C.rep_base + P.r2t[c.rg]];
    float2 zm[NC], zc[NC];
    const uint32_t zmb = (c.z0 == 0 ? L - 1 : c.z0 - 1) * c.Pz;
    float lx[NC];
    float2 lyp[NC], lym[NC], lzp[NC], lv[NC];
    auto ld2 = [](const float* q) { return __ldg(reinterpret_cast<const float2*>(q)); };
    auto load_step = [&](uint32_t z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t zb = z * c.Pz, zpb = (z + 1 == L ? 0 : z + 1) * c.Pz;
        const uint32_t xo = p ? xo1 : xo0;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float* o = oth + (size_t)k * plane;
            lx[k] = __ldg(o + zb + xo);
            lyp[k] = ld2(o + zb + colp);
            lym[k] = ld2(o + zb + colm);
            lzp[k] = ld2(o + zpb + c.col);
            lv[k] = *reinterpret_cast<const float2*>(own + (size_t)k * plane + zb + c.col);
        }
    };
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        zm[k] = ld2(oth + (size_t)k * plane + zmb + c.col);
        zc[k] = ld2(oth + (size_t)k * plane + c.z0 * c.Pz + c.col);
    }
    load_step(c.z0);
    for (uint32_t z = c.z0; z < c.z1; ++z) {
        const uint32_t p = (c.y + z + (uint32_t)colour) & 1u;
        const uint32_t i = z * c.Pz + c.col;  // site k; site k+1 is i + 1
        float ha[NC], hb[NC], va[NC], vb[NC], wa[NC], wb[NC];
        float na[6][NC], nb[6][NC];
        float2 zp[NC];
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float xn = lx[k];
            const float xpa = p ? zc[k].y : zc[k].x, xma = p ? zc[k].x : xn;
            const float xpb = p ? xn : zc[k].y, xmb = p ? zc[k].y : zc[k].x;
            zp[k] = lzp[k];
            ha[k] = ((xpa + xma) + (lyp[k].x + lym[k].x)) + (zp[k].x + zm[k].x);
            hb[k] = ((xpb + xmb) + (lyp[k].y + lym[k].y)) + (zp[k].y + zm[k].y);
            va[k] = lv[k].x;
            vb[k] = lv[k].y;
            if (MEAS) {
                na[0][k] = xpa;
                na[1][k] = xma;
                na[2][k] = lyp[k].x;
                na[3][k] = lym[k].x;
                na[4][k] = zp[k].x;
                na[5][k] = zm[k].x;
                nb[0][k] = xpb;
                nb[1][k] = xmb;
                nb[2][k] = lyp[k].y;
                nb[3][k] = lym[k].y;
                nb[4][k] = zp[k].y;
                nb[5][k] = zm[k].y;
            }
        }
        if (z + 1 < c.z1) load_step(z + 1);
        // O(3): one block per site; O(2): the pair's one block (i is even),
        // words (x, z) for site k, (y, w) for site k+1
        U4 u0, u1;
        if constexpr (NC == 3) {
            u0 = philox_w(pre, P, i);
            u1 = philox_w(pre, P, i + 1);
        } else {
            u0 = philox_w(pre, P, i >> 1);
            u1 = U4{u0.y, u0.x, u0.w, u0.z};
        }
        const bool acc_a = cone_test<NC>(va, ha, u0, cos_delta, delta, beta, P.J, wa);
        const bool acc_b = cone_test<NC>(vb, hb, u1, cos_delta, delta, beta, P.J, wb);
        n_acc += (acc_a ? 1u : 0u) + (acc_b ? 1u : 0u);
        const bool wr_a = acc_a || renorm_now, wr_b = acc_b || renorm_now;
        if (MEAS || wr_a || wr_b) {
            float n2a = 0.f, n2b = 0.f;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                if (acc_a) va[k] = wa[k];
                if (acc_b) vb[k] = wb[k];
                n2a = fmaf(va[k], va[k], n2a);
                n2b = fmaf(vb[k], vb[k], n2b);
            }
            const float sca = renorm_now ? rsqrtf(n2a) : 1.0f;
            const float scb = renorm_now ? rsqrtf(n2b) : 1.0f;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                va[k] = wr_a ? va[k] * sca : va[k];
                vb[k] = wr_b ? vb[k] * scb : vb[k];
            }
            if (wr_a || wr_b) {
#pragma unroll
                for (int k = 0; k < NC; ++k)
                    *reinterpret_cast<float2*>(own + (size_t)k * plane + i) = make_float2(va[k], vb[k]);
            }
        }
        if (MEAS) {
#pragma unroll
            for (int k = 0; k < NC; ++k) acc[1 + k] += fx(va[k]) + fx(zc[k].x);
            meas_bonds<NC>(acc, va, na);
#pragma unroll
            for (int k = 0; k < NC; ++k) acc[1 + k] += fx(vb[k]) + fx(zc[k].y);
            meas_bonds<NC>(acc, vb, nb);
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            zm[k] = zc[k];
            zc[k] = zp[k];
        }
    }
}

__device__ __forceinline__ void count_accepted(const ContParams& P, int rg, unsigned n_acc) {
    // per-replica acceptance count: one atomic per warp when the warp's
    // tasks are of one replica
    const int lane = threadIdx.x & 31;
    const int rg0 = __shfl_sync(ISG_FULL_MASK, rg, 0);
    const unsigned cnt = __reduce_add_sync(ISG_FULL_MASK, n_acc);
    if (__all_sync(ISG_FULL_MASK, rg == rg0 || rg < 0)) {
        if (lane == 0 && rg0 >= 0 && cnt) atomicAdd(&P.metro_acc[rg0], (unsigned long long)cnt);
    } else if (rg >= 0 && n_acc) {
        atomicAdd(&P.metro_acc[rg], (unsigned long long)n_acc);
    }
}

template <int NC>
__global__ void __launch_bounds__(kCThreads, NC == 2 ? 3 : 2)
    k_cont_metro_col2(const __grid_constant__ ContParams P, int colour, int sweep_off,
                      float cos_delta, float delta) {
    const uint64_t sweep = P.ctrl[0] + (uint64_t)sweep_off;
    const bool renorm_now = P.renorm > 0 && ((sweep + 1) % (uint64_t)P.renorm) == 0;
    const uint32_t c2 = (uint32_t)sweep;
    const uint32_t c3 = counter_word3(ISG_TAG_CMETRO, (uint32_t)colour, sweep);
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    ColRef c;
    const bool live = col_locate(P, 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x), c);
    unsigned n_acc = 0;
    int none[kNQ];
    if (live)
        metro2_column<NC, false>(P, c, colour, c2, c3, k0, k1, cos_delta, delta, renorm_now,
                                 n_acc, none);
    count_accepted(P, live ? c.rg : -1, n_acc);
}

// The colour-1 Metropolis half-sweep of a measured sweep with the measurement
// fused in: blocks are the measurement chunks of k_cont_measure2 (kCThreads
// two-site column tasks of one replica), and each block stores its partials
// for k_cont_combine.  The spins are updated exactly as by k_cont_metro_col2
// (the random stream is defined per site), and the 10 sums equal
// k_cont_measure2's on the updated spins, so this replaces the pair
// "Metropolis colour 1, then measure" and saves the measurement's pass over
// both colour planes.
template <int NC>
__global__ void __launch_bounds__(kCThreads, 2)
    k_cont_metro_meas2(const __grid_constant__ ContParams P, int sweep_off, float cos_delta,
                       float delta) {
    const uint64_t sweep = P.ctrl[0] + (uint64_t)sweep_off;
    const bool renorm_now = P.renorm > 0 && ((sweep + 1) % (uint64_t)P.renorm) == 0;
    const uint32_t c2 = (uint32_t)sweep;
    const uint32_t c3 = counter_word3(ISG_TAG_CMETRO, 1u, sweep);
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const int chunk = blockIdx.x;
    int ci = 0;
    while (ci + 1 < P.n_classes && P.cls[ci + 1].chunk_base <= chunk) ++ci;
    const ContClass& C = P.cls[ci];
    const int lc = chunk - C.chunk_base;
    const int r = lc / C.chunks_per_rep;
    const uint32_t L = (uint32_t)C.L, half = L >> 1, Pz = L * half;
    const uint32_t u = (uint32_t)(lc - r * C.chunks_per_rep) * kCThreads + threadIdx.x;
    int acc[kNQ];
#pragma unroll
    for (int q = 0; q < kNQ; ++q) acc[q] = 0;
    unsigned n_acc = 0;
    const bool live = u < (uint32_t)C.nseg * (Pz / 2);
    if (live) {
        ColRef c;
        const uint32_t zseg = u / (Pz / 2);
        c.ci = ci;
        c.r = r;
        c.rg = C.rep_base + r;
        c.Pz = Pz;
        c.col = 2 * (u - zseg * (Pz / 2));
        c.y = fdiv(c.col, C.div_half);
        c.k = c.col - c.y * half;
        c.z0 = zseg * kColZ;
        c.z1 = min(L, c.z0 + (uint32_t)kColZ);
        metro2_column<NC, true>(P, c, 1, c2, c3, k0, k1, cos_delta, delta, renorm_now, n_acc,
                                acc);
    }
    count_accepted(P, live ? C.rep_base + r : -1, n_acc);
    meas_block_store(P, acc, chunk);
}

// Block reduction of the fixed-point sums into one int64 partial per quantity
// (slot 0, the energy, is formed at the combine).  A thread's sums are below
// 2^30, so a warp sums their upper parts (>> 8) and low bytes separately in
// int32 and joins them in int64.
__device__ __forceinline__ void meas_block_store(const ContParams& P, int (&acc)[kNQ], int chunk) {
    __shared__ long long red[kCThreads / 32][kNQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 1; q < kNQ; ++q) {
        const int hi = __reduce_add_sync(ISG_FULL_MASK, acc[q] >> 8);
        const unsigned lo = __reduce_add_sync(ISG_FULL_MASK, (unsigned)(acc[q] & 0xFF));
        if (lane == 0) red[wid][q] = (long long)hi * 256 + (long long)lo;
    }
    __syncthreads();
    if (threadIdx.x < kNQ) {
        long long v = 0;
        if (threadIdx.x > 0)
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        P.partials[(int64_t)chunk * kNQ + threadIdx.x] = v;
    }
}

// Per block: kCThreads column tasks of one replica (chunks_per_rep blocks per
// replica; two-site tasks in k_cont_measure2), each walking up to kColZ
// z-planes of colour-1 sites.  Each
// colour-1 site owns its six bonds (every bond has exactly one colour-1 end)
// and, for M, its colour-0 partner at the same colour index.  The summation
// order is fixed by the task layout, so the result is deterministic.
template <int NC>
__global__ void __launch_bounds__(kCThreads) k_cont_measure(const __grid_constant__ ContParams P) {
    const int chunk = blockIdx.x;
    int ci = 0;
    while (ci + 1 < P.n_classes && P.cls[ci + 1].chunk_base <= chunk) ++ci;
    const ContClass& C = P.cls[ci];
    const int lc = chunk - C.chunk_base;
    const int r = lc / C.chunks_per_rep;
    const uint32_t L = (uint32_t)C.L, half = L >> 1, Pz = L * half, plane = C.plane_sites;
    const uint32_t u = (uint32_t)(lc - r * C.chunks_per_rep) * kCThreads + threadIdx.x;
    int acc[kNQ];
#pragma unroll
    for (int q = 0; q < kNQ; ++q) acc[q] = 0;
    if (u < (uint32_t)C.nseg * Pz) {
        const uint32_t zseg = u / Pz, col = u - zseg * Pz;
        const uint32_t y = fdiv(col, C.div_half), k = col - y * half;
        const uint32_t z0 = zseg * kColZ, z1 = min(L, z0 + (uint32_t)kColZ);
        const float* own = P.spins + plane_off<NC>(C, r, 1, 0);
        const float* oth = P.spins + plane_off<NC>(C, r, 0, 0);
        const uint32_t row = y * half;
        const uint32_t xo1 = row + (k + 1 == half ? 0 : k + 1);
        const uint32_t xo0 = row + (k == 0 ? half - 1 : k - 1);
        const uint32_t colp = (y + 1 == L ? 0 : y + 1) * half + k;
        const uint32_t colm = (y == 0 ? L - 1 : y - 1) * half + k;
        float zm[NC], zc[NC];
        const uint32_t zmb = (z0 == 0 ? L - 1 : z0 - 1) * Pz;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            zm[c] = __ldg(oth + (size_t)c * plane + zmb + col);
            zc[c] = __ldg(oth + (size_t)c * plane + z0 * Pz + col);
        }
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t p = (y + z + 1u) & 1u;
            const uint32_t zb = z * Pz, zpb = (z + 1 == L ? 0 : z + 1) * Pz;
            const uint32_t xo = p ? xo1 : xo0;
            float s[NC], n[6][NC], zp[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const float* o = oth + (size_t)c * plane;
                const float xn = __ldg(o + zb + xo);
                n[2][c] = __ldg(o + zb + colp);
                n[3][c] = __ldg(o + zb + colm);
                zp[c] = __ldg(o + zpb + col);
                s[c] = __ldg(own + (size_t)c * plane + zb + col);
                n[0][c] = p ? xn : zc[c];
                n[1][c] = p ? zc[c] : xn;
                n[4][c] = zp[c];
                n[5][c] = zm[c];
                acc[1 + c] += fx(s[c]) + fx(zc[c]);
            }
            meas_bonds<NC>(acc, s, n);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                zm[c] = zc[c];
                zc[c] = zp[c];
            }
        }
    }
    meas_block_store(P, acc, chunk);
}

// The same measurement with two adjacent colour-1 sites (k, k+1 of a row)
// per thread, for batches whose sizes are all multiples of 4: 64-bit loads,
// and the block reduction spread over twice the sites.  Per z the thread adds
// site k's terms, then site k+1's.
template <int NC>
__global__ void __launch_bounds__(kCThreads, 3) k_cont_measure2(const __grid_constant__ ContParams P) {
    const int chunk = blockIdx.x;
    int ci = 0;
    while (ci + 1 < P.n_classes && P.cls[ci + 1].chunk_base <= chunk) ++ci;
    const ContClass& C = P.cls[ci];
    const int lc = chunk - C.chunk_base;
    const int r = lc / C.chunks_per_rep;
    const uint32_t L = (uint32_t)C.L, half = L >> 1, Pz = L * half, plane = C.plane_sites;
    const uint32_t u = (uint32_t)(lc - r * C.chunks_per_rep) * kCThreads + threadIdx.x;
    int acc[kNQ];
#pragma unroll
    for (int q = 0; q < kNQ; ++q) acc[q] = 0;
    if (u < (uint32_t)C.nseg * (Pz / 2)) {
        const uint32_t zseg = u / (Pz / 2), col = 2 * (u - zseg * (Pz / 2));
        const uint32_t y = fdiv(col, C.div_half), k = col - y * half;
        const uint32_t z0 = zseg * kColZ, z1 = min(L, z0 + (uint32_t)kColZ);
        const float* own = P.spins + plane_off<NC>(C, r, 1, 0);
        const float* oth = P.spins + plane_off<NC>(C, r, 0, 0);
        const uint32_t row = y * half;
        const uint32_t xo1 = row + (k + 2 == half ? 0 : k + 2);  // x+ of site k+1 (p = 1)
        const uint32_t xo0 = row + (k == 0 ? half - 1 : k - 1);  // x- of site k (p = 0)
        const uint32_t colp = (y + 1 == L ? 0 : y + 1) * half + k;
        const uint32_t colm = (y == 0 ? L - 1 : y - 1) * half + k;
        auto ld2 = [](const float* q) { return __ldg(reinterpret_cast<const float2*>(q)); };
        float2 zm[NC], zc[NC];
        const uint32_t zmb = (z0 == 0 ? L - 1 : z0 - 1) * Pz;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            zm[c] = ld2(oth + (size_t)c * plane + zmb + col);
            zc[c] = ld2(oth + (size_t)c * plane + z0 * Pz + col);
        }
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t p = (y + z + 1u) & 1u;
            const uint32_t zb = z * Pz, zpb = (z + 1 == L ? 0 : z + 1) * Pz;
            const uint32_t xo = p ? xo1 : xo0;
            float sa[NC], sb[NC], na[6][NC], nb[6][NC];
            float2 zp[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const float* o = oth + (size_t)c * plane;
                const float xn = __ldg(o + zb + xo);
                const float2 yp = ld2(o + zb + colp), ym = ld2(o + zb + colm);
                zp[c] = ld2(o + zpb + col);
                const float2 sv = ld2(own + (size_t)c * plane + zb + col);
                sa[c] = sv.x;
                sb[c] = sv.y;
                na[0][c] = p ? zc[c].y : zc[c].x;
                na[1][c] = p ? zc[c].x : xn;
                nb[0][c] = p ? xn : zc[c].y;
                nb[1][c] = p ? zc[c].y : zc[c].x;
                na[2][c] = yp.x;
                nb[2][c] = yp.y;
                na[3][c] = ym.x;
                nb[3][c] = ym.y;
                na[4][c] = zp[c].x;
                nb[4][c] = zp[c].y;
                na[5][c] = zm[c].x;
                nb[5][c] = zm[c].y;
            }
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[1 + c] += fx(sa[c]) + fx(zc[c].x);
            meas_bonds<NC>(acc, sa, na);
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[1 + c] += fx(sb[c]) + fx(zc[c].y);
            meas_bonds<NC>(acc, sb, nb);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                zm[c] = zc[c];
                zc[c] = zp[c];
            }
        }
    }
    meas_block_store(P, acc, chunk);
}

// Combine of the block partials of each replica: exact int64 sums, then
// one conversion to FP64 (units of 2^-24); E = -J (C_x + C_y + C_z).
__global__ void k_cont_combine(const __grid_constant__ ContParams P, double* out) {
    const int rg = blockIdx.x * blockDim.x + threadIdx.x;
    int ci = 0;
    while (ci + 1 < P.n_classes && P.cls[ci + 1].rep_base <= rg) ++ci;
    const ContClass& C = P.cls[ci];
    if (rg >= C.rep_base + C.R) return;
    const int r = rg - C.rep_base;
    long long q[kNQ];
    for (int k = 0; k < kNQ; ++k) q[k] = 0;
    const int c0 = C.chunk_base + r * C.chunks_per_rep;
    for (int c = 0; c < C.chunks_per_rep; ++c)
        for (int k = 1; k < kNQ; ++k) q[k] += P.partials[(int64_t)(c0 + c) * kNQ + k];
    const double unit = 1.0 / 16777216.0;
    out[(int64_t)rg * kNQ] = __dmul_rn(-P.Jd, (double)(q[4] + q[5] + q[6]) * unit);
    for (int k = 1; k < kNQ; ++k) out[(int64_t)rg * kNQ + k] = (double)q[k] * unit;
}

__global__ void k_cont_init(const __grid_constant__ ContParams P, int nc) {
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const uint32_t c3 = counter_word3(ISG_TAG_CINIT, 0, 0);
    for (int ci = 0; ci < P.n_classes; ++ci) {
        const ContClass& C = P.cls[ci];
        const int64_t nsite = 2 * (int64_t)C.plane_sites;
        const int64_t total = nsite * C.R;
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
             g += (int64_t)gridDim.x * blockDim.x) {
            const int r = (int)(g / nsite);
            const uint32_t n = (uint32_t)(g - (int64_t)r * nsite);
            const U4 u = philox10(replica_uid(C.L, r), n, 0, c3, k0, k1);
            const uint32_t L = (uint32_t)C.L;
            const uint32_t x = n % L, y = (n / L) % L, z = n / (L * L);
            const int c = (int)((x + y + z) & 1u);
            float v[3];
            if (nc == 3) {
                // z uniform in [-1, 1), phi uniform in [0, 2pi): uniform on S^2
                const float zz = 2.0f * uniform24(u.x) - 1.0f;
                float sp, cp;
                sincospif(2.0f * uniform24(u.y), &sp, &cp);
                const float rr = sqrtf(fmaxf(0.0f, 1.0f - zz * zz));
                v[0] = rr * cp;
                v[1] = rr * sp;
                v[2] = zz;
            } else {
                sincospif(2.0f * uniform24(u.x), &v[1], &v[0]);
                v[2] = 0.f;
            }
            for (int k = 0; k < nc; ++k) {
                const int64_t o = C.off + (int64_t)r * 2 * nc * C.plane_sites +
                                  (int64_t)(c * nc + k) * C.plane_sites + (n >> 1);
                P.spins[o] = v[k];
            }
        }
    }
}

__global__ void k_cont_normalize(const __grid_constant__ ContParams P, int nc) {
    for (int ci = 0; ci < P.n_classes; ++ci) {
        const ContClass& C = P.cls[ci];
        const int64_t total = 2 * (int64_t)C.plane_sites * C.R;
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
             g += (int64_t)gridDim.x * blockDim.x) {
            const int64_t rc = g / C.plane_sites;  // replica*2 + colour
            const int64_t i = g - rc * C.plane_sites;
            float* b = P.spins + C.off + rc * nc * C.plane_sites + i;
            float n2 = 0.f;
            for (int k = 0; k < nc; ++k) n2 = fmaf(b[k * C.plane_sites], b[k * C.plane_sites], n2);
            const float sc = rsqrtf(n2);
            for (int k = 0; k < nc; ++k) b[k * C.plane_sites] *= sc;
        }
    }
}

struct ContPost {
    const double* obs;  // [replicas][kNQ]
    int32_t* r2t;
    int32_t* t2r;
    const double* betas;
    int32_t* rec_t;
    double* rec_e;
    double* rec_m;  // [cap][RT][3]
    double* rec_h;  // [cap][RT][6]
    unsigned long long* ctrl;
    long long ring_cap;
    uint64_t seed;
    int R, n_classes, replicas_total;
    int L[kCMaxClasses];
};

__global__ void k_cont_post(const __grid_constant__ ContPost Q, int do_record, int do_exchange,
                            int parity, int advance) {
    __shared__ double s_e[kCMaxReplicas];
    __shared__ int s_t2r[kCMaxReplicas];
    __shared__ int s_acc;
    const int s = blockIdx.x;
    const int R = Q.R, base = s * R, NC = Q.n_classes;
    unsigned long long* rec_count = Q.ctrl + 1 + s;
    unsigned long long* xcount = Q.ctrl + 1 + NC + s;
    unsigned long long* accepted = Q.ctrl + 1 + 2 * NC + s;
    if (threadIdx.x == 0) s_acc = 0;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const double* o = Q.obs + (int64_t)(base + r) * kNQ;
        s_e[r] = o[0];
        s_t2r[r] = Q.t2r[base + r];
        if (do_record) {
            const long long slot = (long long)(*rec_count % (unsigned long long)Q.ring_cap);
            const long long idx = slot * Q.replicas_total + base + r;
            Q.rec_t[idx] = Q.r2t[base + r];
            Q.rec_e[idx] = o[0];
            for (int k = 0; k < 3; ++k) Q.rec_m[idx * 3 + k] = o[1 + k];
            for (int k = 0; k < 6; ++k) Q.rec_h[idx * 6 + k] = o[4 + k];
        }
    }
    __syncthreads();
    if (do_exchange) {
        const unsigned long long xc = *xcount;
        const int par = parity >= 0 ? (parity & 1) : (int)(xc & 1ull);
        const uint32_t k0 = (uint32_t)Q.seed, k1 = (uint32_t)(Q.seed >> 32);
        const uint32_t c3 = counter_word3(ISG_TAG_EXCH, 0, xc);
        for (int i = par + 2 * threadIdx.x; i + 1 < R; i += 2 * blockDim.x) {
            const int ri = s_t2r[i], rj = s_t2r[i + 1];
            const double d = __dmul_rn(__dsub_rn(Q.betas[base + i], Q.betas[base + i + 1]),
                                       __dsub_rn(s_e[rj], s_e[ri]));
            bool ok = d < 0.0;
            if (!ok) {
                const U4 u = philox10(exchange_uid(Q.L[s]), (uint32_t)i, (uint32_t)xc, c3, k0, k1);
                ok = uniform53(u.x, u.y) < exp(-d);
            }
            if (ok) {
                s_t2r[i] = rj;
                s_t2r[i + 1] = ri;
                Q.r2t[base + ri] = i + 1;
                Q.r2t[base + rj] = i;
                atomicAdd(&s_acc, 1);
            }
        }
        __syncthreads();
        for (int r = threadIdx.x; r < R; r += blockDim.x) Q.t2r[base + r] = s_t2r[r];
        if (threadIdx.x == 0) {
            *xcount = xc + 1;
            *accepted += (unsigned long long)s_acc;
        }
    }
    if (threadIdx.x == 0) {
        if (do_record) *rec_count += 1ull;
        if (s == 0 && advance) Q.ctrl[0] += (unsigned long long)advance;
    }
}

}  // namespace isg

using namespace isg;

struct isg_cont {
    int device = 0;
    int nc = 3;
    int n_classes = 0;
    int R = 0;
    int RT = 0;
    uint64_t seed = 0;
    std::vector<int> sizes;
    ContParams P{};
    ContPost Q{};
    float* d_spins = nullptr;
    int64_t n_floats = 0;
    float* d_betaf = nullptr;
    double* d_betas = nullptr;
    int32_t* d_r2t = nullptr;
    int32_t* d_t2r = nullptr;
    unsigned long long* d_ctrl = nullptr;
    unsigned long long* d_macc = nullptr;
    long long* d_partials = nullptr;
    double* d_obs = nullptr;
    int64_t ring_cap = 0;
    unsigned char* h_stage = nullptr;  // pinned staging of drained records
    int32_t* d_rec_t = nullptr;
    double* d_rec_e = nullptr;
    double* d_rec_m = nullptr;
    double* d_rec_h = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    bool temps_set = false;
    double J = 1.0;
    int sms = 1;
    int grid = 1;
    bool pairs = false;  // every size a multiple of 4: two-site column kernels
    bool fuse_measure = true;  // measured sweeps: measurement fused into the last half-sweep
    uint64_t ksample = 0, records_made = 0, records_done = 0;
    cudaGraphExec_t graph = nullptr;
    int g_ee = 0, g_me = 0, g_period = 0, g_nor = -1, g_renorm = -1;
    double g_delta = -1.0;
};

namespace isg {

static void cont_destroy_graph(isg_cont* H) {
    if (H->graph) cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
    H->g_period = 0;
}

static void launch_or(isg_cont* H, int colour) {
    if (H->pairs) {
        const int64_t n = H->P.total_cols / 2;
        const unsigned g2 = (unsigned)((n + kCThreads - 1) / kCThreads);
        if (H->nc == 3)
            k_cont_or_col2<3><<<g2, kCThreads, 0, H->stream>>>(H->P, colour);
        else
            k_cont_or_ring2<2><<<g2, kCThreads, or_ring_bytes<2>(), H->stream>>>(H->P, colour);
        return;
    }
    const unsigned grid = (unsigned)((H->P.total_cols + kCThreads - 1) / kCThreads);
    if (H->nc == 3)
        k_cont_or_col<3><<<grid, kCThreads, 0, H->stream>>>(H->P, colour);
    else
        k_cont_or_col<2><<<grid, kCThreads, 0, H->stream>>>(H->P, colour);
}

static void launch_metro(isg_cont* H, int colour, int sweep_off, double delta) {
    const float cd = (float)std::cos(std::min(delta, M_PI));
    if (H->pairs) {
        const int64_t n = H->P.total_cols / 2;
        const unsigned g2 = (unsigned)((n + kCThreads - 1) / kCThreads);
        if (H->nc == 3)
            k_cont_metro_col2<3><<<g2, kCThreads, 0, H->stream>>>(H->P, colour, sweep_off, cd,
                                                                  (float)delta);
        else
            k_cont_metro_col2<2><<<g2, kCThreads, 0, H->stream>>>(H->P, colour, sweep_off, cd,
                                                                  (float)delta);
        return;
    }
    const unsigned grid = (unsigned)((H->P.total_cols + kCThreads - 1) / kCThreads);
    if (H->nc == 3)
        k_cont_metro_col<3><<<grid, kCThreads, 0, H->stream>>>(H->P, colour, sweep_off, cd,
                                                               (float)delta);
    else
        k_cont_metro_col<2><<<grid, kCThreads, 0, H->stream>>>(H->P, colour, sweep_off, cd,
                                                               (float)delta);
}

static void launch_measure(isg_cont* H) {
    if (H->pairs) {
        if (H->nc == 3)
            k_cont_measure2<3><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P);
        else
            k_cont_measure2<2><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P);
        k_cont_combine<<<(H->RT + 127) / 128, 128, 0, H->stream>>>(H->P, H->d_obs);
        return;
    }
    if (H->nc == 3)
        k_cont_measure<3><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P);
    else
        k_cont_measure<2><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P);
    k_cont_combine<<<(H->RT + 127) / 128, 128, 0, H->stream>>>(H->P, H->d_obs);
}

static void launch_cpost(isg_cont* H, int rec, int xch, int parity, int advance) {
    const int thr = std::min(1024, std::max(32, ((H->R + 31) / 32) * 32));
    k_cont_post<<<H->n_classes, thr, 0, H->stream>>>(H->Q, rec, xch, parity, advance);
}

// One sweep in the reference GPU order: n_or overrelaxation sweeps, then one
// Metropolis sweep (gpu_lattice_continuous.rs:123-168).
static void issue_cont_sweep(isg_cont* H, int sweep_off, double delta, int n_or) {
    for (int k = 0; k < n_or; ++k) {
        launch_or(H, 0);
        launch_or(H, 1);
    }
    launch_metro(H, 0, sweep_off, delta);
    launch_metro(H, 1, sweep_off, delta);
}

// The colour-1 Metropolis half-sweep with the measurement fused in (two-site
// column batches), then the FP64 combine of the block partials.
static void launch_metro_measure(isg_cont* H, int sweep_off, double delta) {
    const float cd = (float)std::cos(std::min(delta, M_PI));
    if (H->nc == 3)
        k_cont_metro_meas2<3><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P, sweep_off, cd,
                                                                              (float)delta);
    else
        k_cont_metro_meas2<2><<<H->P.total_chunks, kCThreads, 0, H->stream>>>(H->P, sweep_off, cd,
                                                                              (float)delta);
    k_cont_combine<<<(H->RT + 127) / 128, 128, 0, H->stream>>>(H->P, H->d_obs);
}

static void issue_cont_sample(isg_cont* H, uint64_t k, int sweep_off, int ee, int me,
                              double delta, int n_or, int advance) {
    const bool do_m = ((k + 1) % (uint64_t)me) == 0;
    const bool do_x = ((k + 1) % (uint64_t)ee) == 0;
    if ((do_m || do_x) && H->pairs && H->fuse_measure) {
        // measured sweep: the measurement rides on the last half-sweep
        for (int j = 0; j < n_or; ++j) {
            launch_or(H, 0);
            launch_or(H, 1);
        }
        launch_metro(H, 0, sweep_off, delta);
        launch_metro_measure(H, sweep_off, delta);
    } else {
        issue_cont_sweep(H, sweep_off, delta, n_or);
        if (do_m || do_x) launch_measure(H);
    }
    if (do_m || do_x || advance) launch_cpost(H, do_m ? 1 : 0, do_x ? 1 : 0, -1, advance);
}

static int cont_check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return ISG_OK;
}

// Records leave the device ring through a pinned staging buffer of at most
// 4 MiB: each batch's copies (at most two ring chunks per array) are queued
// on the stream behind the sweeps that made them, the host waits once, then
// copies the rows into the caller's arrays.
static int cont_drain(isg_cont* H, int32_t* t, double* e, double* m, double* hb, int64_t row0) {
    const int RT = H->RT;
    uint64_t n = H->records_made - H->records_done;
    if (n == 0) {
        ISG_CK(cudaStreamSynchronize(H->stream));
        return ISG_OK;
    }
    constexpr size_t kRowBytes = 4 + 8 + 3 * 8 + 6 * 8;  // per replica: slot, E, M[3], bonds[6]
    const uint64_t srows =
        std::max<uint64_t>(1, std::min<uint64_t>(256, ((size_t)4 << 20) / (kRowBytes * RT)));
    const size_t sn = (size_t)srows * RT;
    if (!H->h_stage) ISG_CK(cudaMallocHost((void**)&H->h_stage, sn * kRowBytes));
    double* st_e = reinterpret_cast<double*>(H->h_stage);
    double* st_m = st_e + sn;
    double* st_h = st_m + 3 * sn;
    int32_t* st_t = reinterpret_cast<int32_t*>(st_h + 6 * sn);
    int64_t row = row0;
    while (n > 0) {
        const uint64_t batch = std::min<uint64_t>(n, srows);
        uint64_t done = H->records_done, left = batch;
        size_t srow = 0;
        while (left > 0) {
            const uint64_t slot = done % (uint64_t)H->ring_cap;
            const uint64_t chunk = std::min<uint64_t>(left, (uint64_t)H->ring_cap - slot);
            const size_t cnt = (size_t)chunk * RT, off = (size_t)slot * RT, so = srow * RT;
            ISG_CK(cudaMemcpyAsync(st_t + so, H->d_rec_t + off, cnt * sizeof(int32_t),
                                   cudaMemcpyDeviceToHost, H->stream));
            ISG_CK(cudaMemcpyAsync(st_e + so, H->d_rec_e + off, cnt * sizeof(double),
                                   cudaMemcpyDeviceToHost, H->stream));
            ISG_CK(cudaMemcpyAsync(st_m + so * 3, H->d_rec_m + off * 3, cnt * 3 * sizeof(double),
                                   cudaMemcpyDeviceToHost, H->stream));
            ISG_CK(cudaMemcpyAsync(st_h + so * 6, H->d_rec_h + off * 6, cnt * 6 * sizeof(double),
                                   cudaMemcpyDeviceToHost, H->stream));
            srow += chunk;
            done += chunk;
            left -= chunk;
        }
        ISG_CK(cudaStreamSynchronize(H->stream));
        const size_t cnt = (size_t)batch * RT;
        memcpy(t + (size_t)row * RT, st_t, cnt * sizeof(int32_t));
        memcpy(e + (size_t)row * RT, st_e, cnt * sizeof(double));
        memcpy(m + (size_t)row * RT * 3, st_m, cnt * 3 * sizeof(double));
        memcpy(hb + (size_t)row * RT * 6, st_h, cnt * 6 * sizeof(double));
        H->records_done += batch;
        row += (int64_t)batch;
        n -= batch;
    }
    return ISG_OK;
}

}  // namespace isg

extern "C" {

int isg_cont_create(isg_cont** out, const int* sizes, int n_sizes, int replicas, int n_comp,
                    uint64_t seed) {
    if (!out) return fail(ISG_ERR_ARG, "isg_cont_create: out is NULL");
    *out = nullptr;
    if (!sizes || n_sizes < 1 || n_sizes > kCMaxClasses)
        return fail(ISG_ERR_ARG, "isg_cont_create: need 1..16 sizes");
    if (replicas < 1 || replicas > kCMaxReplicas)
        return fail(ISG_ERR_ARG, "isg_cont_create: replicas must be 1..1024");
    if (n_comp != 2 && n_comp != 3)
        return fail(ISG_ERR_ARG, "isg_cont_create: n_comp must be 2 (XY) or 3 (Heisenberg)");
    for (int s = 0; s < n_sizes; ++s) {
        const int L = sizes[s];
        if (L < 2 || L > 1024)
            return fail(ISG_ERR_ARG, "isg_cont_create: size " + std::to_string(L) +
                                         " outside 2..1024");
        for (int q = 0; q < s; ++q)
            if (sizes[q] == L)
                return fail(ISG_ERR_ARG, "isg_cont_create: size " + std::to_string(L) +
                                             " listed twice (sizes share random streams)");
        if (L & 1)
            return fail(ISG_ERR_UNSUPPORTED,
                        "isg_cont_create: odd size " + std::to_string(L) +
                            " has no checkerboard colouring under periodic boundaries");
    }
    isg_cont* H = new (std::nothrow) isg_cont();
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_create: out of host memory");
    cudaGetDevice(&H->device);
    cudaDeviceGetAttribute(&H->sms, cudaDevAttrMultiProcessorCount, H->device);
    if (H->sms < 1) H->sms = 1;
    {
        // the O(2) overrelaxation ring exceeds the 48 KB default
        const cudaError_t a = cudaFuncSetAttribute(
            k_cont_or_ring2<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)or_ring_bytes<2>());
        if (a != cudaSuccess) {
            delete H;
            return cuda_fail(a, "isg_cont_create: cudaFuncSetAttribute");
        }
    }
    H->nc = n_comp;
    H->n_classes = n_sizes;
    H->R = replicas;
    H->RT = n_sizes * replicas;
    H->seed = seed;
    H->sizes.assign(sizes, sizes + n_sizes);
    ContParams& P = H->P;
    int64_t off = 0, site = 0;
    int chunk = 0;
    P.total_cols = 0;
    H->pairs = true;
    for (int s = 0; s < n_sizes; ++s)
        if (sizes[s] % 4 != 0) H->pairs = false;
    const int64_t per_task = H->pairs ? 2 : 1;  // column tasks per measurement thread
    for (int s = 0; s < n_sizes; ++s) {
        ContClass& C = P.cls[s];
        const int L = sizes[s];
        C.L = L;
        C.R = replicas;
        C.plane_sites = (uint32_t)((int64_t)L * L * L / 2);
        C.div_half = make_div((uint32_t)(L / 2));
        C.div_L = make_div((uint32_t)L);
        C.div_plane = make_div(C.plane_sites);
        C.small = (int64_t)C.plane_sites * replicas < (1ll << 31) ? 1 : 0;
        C.rep_base = s * replicas;
        C.nseg = (L + kColZ - 1) / kColZ;
        C.col_base = P.total_cols;
        P.total_cols += (int64_t)replicas * C.nseg * ((int64_t)L * L / 2);
        C.col_end = P.total_cols;
        C.off = off;
        off += ((2 * (int64_t)n_comp * C.plane_sites * replicas + 63) / 64) * 64;
        C.site_base = site;
        site += (int64_t)C.plane_sites * replicas;
        C.site_end = site;
        C.chunks_per_rep = (int)(((int64_t)C.nseg * ((int64_t)L * L / 2) / per_task + kCThreads - 1) /
                                 kCThreads);
        C.chunk_base = chunk;
        chunk += C.chunks_per_rep * replicas;
    }
    for (int s = n_sizes; s < kCMaxClasses; ++s) {
        P.cls[s] = P.cls[n_sizes - 1];
        P.cls[s].site_base = P.cls[s].site_end = INT64_MAX;
        P.cls[s].col_base = P.cls[s].col_end = INT64_MAX;
        P.cls[s].chunk_base = INT32_MAX;
        P.cls[s].rep_base = INT32_MAX;
    }
    P.n_classes = n_sizes;
    P.total_sites = site;
    P.total_chunks = chunk;
    P.seed = seed;
    for (int r = 0; r < 10; ++r) {
        P.rk0[r] = (uint32_t)seed + (uint32_t)r * kPhiloxW0;
        P.rk1[r] = (uint32_t)(seed >> 32) + (uint32_t)r * kPhiloxW1;
    }
    P.J = 1.0f;
    P.Jd = 1.0;
    P.renorm = 0;
    H->n_floats = off;
    const int RT = H->RT;
    H->ring_cap = std::max<int64_t>(64, std::min<int64_t>(8192, (64ll << 20) / (84ll * RT)));
    H->grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)H->sms * 8,
                                                          (site + kCThreads - 1) / kCThreads));
    auto cleanup = [&](int code) {
        isg_cont_destroy(H);
        return code;
    };
    cudaError_t e;
#define ALLOC(ptr, bytes)                                              \
    e = cudaMalloc((void**)&(ptr), (bytes));                           \
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMalloc"));
    ALLOC(H->d_spins, sizeof(float) * (size_t)off);
    ALLOC(H->d_betaf, sizeof(float) * RT);
    ALLOC(H->d_betas, sizeof(double) * RT);
    ALLOC(H->d_r2t, sizeof(int32_t) * RT);
    ALLOC(H->d_t2r, sizeof(int32_t) * RT);
    ALLOC(H->d_ctrl, sizeof(unsigned long long) * (1 + 3 * kCMaxClasses));
    ALLOC(H->d_macc, sizeof(unsigned long long) * RT);
    ALLOC(H->d_partials, sizeof(long long) * (size_t)chunk * kNQ);
    ALLOC(H->d_obs, sizeof(double) * (size_t)RT * kNQ);
    ALLOC(H->d_rec_t, sizeof(int32_t) * (size_t)H->ring_cap * RT);
    ALLOC(H->d_rec_e, sizeof(double) * (size_t)H->ring_cap * RT);
    ALLOC(H->d_rec_m, sizeof(double) * (size_t)H->ring_cap * RT * 3);
    ALLOC(H->d_rec_h, sizeof(double) * (size_t)H->ring_cap * RT * 6);
#undef ALLOC
    e = cudaStreamCreateWithFlags(&H->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaStreamCreateWithFlags"));
    H->stream = H->own_stream;
    P.spins = H->d_spins;
    P.betaf = H->d_betaf;
    P.r2t = H->d_r2t;
    P.ctrl = H->d_ctrl;
    P.metro_acc = H->d_macc;
    P.partials = H->d_partials;
    ContPost& Q = H->Q;
    Q.obs = H->d_obs;
    Q.r2t = H->d_r2t;
    Q.t2r = H->d_t2r;
    Q.betas = H->d_betas;
    Q.rec_t = H->d_rec_t;
    Q.rec_e = H->d_rec_e;
    Q.rec_m = H->d_rec_m;
    Q.rec_h = H->d_rec_h;
    Q.ctrl = H->d_ctrl;
    Q.ring_cap = H->ring_cap;
    Q.seed = seed;
    Q.R = replicas;
    Q.n_classes = n_sizes;
    Q.replicas_total = RT;
    for (int s = 0; s < kCMaxClasses; ++s) Q.L[s] = s < n_sizes ? sizes[s] : 0;
    std::vector<int32_t> ident(RT);
    for (int i = 0; i < RT; ++i) ident[i] = i % replicas;
#define CKC(call)                                                      \
    e = (call);                                                        \
    if (e != cudaSuccess) return cleanup(cuda_fail(e, #call));
    CKC(cudaMemsetAsync(H->d_spins, 0, sizeof(float) * (size_t)off, H->stream));
    CKC(cudaMemsetAsync(H->d_ctrl, 0, sizeof(unsigned long long) * (1 + 3 * kCMaxClasses),
                        H->stream));
    CKC(cudaMemsetAsync(H->d_macc, 0, sizeof(unsigned long long) * RT, H->stream));
    CKC(cudaMemsetAsync(H->d_obs, 0, sizeof(double) * (size_t)RT * kNQ, H->stream));
    CKC(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                        H->stream));
    CKC(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                        H->stream));
    k_cont_init<<<H->sms * 4, 256, 0, H->stream>>>(H->P, n_comp);
    CKC(cudaGetLastError());
    CKC(cudaStreamSynchronize(H->stream));
#undef CKC
    *out = H;
    return ISG_OK;
}

int isg_cont_destroy(isg_cont* H) {
    if (!H) return ISG_OK;
    cudaSetDevice(H->device);
    // A caller's stream may already be gone: wait for the device instead.
    if (H->stream == H->own_stream) {
        if (H->stream) cudaStreamSynchronize(H->stream);
    } else {
        cudaDeviceSynchronize();
    }
    cont_destroy_graph(H);
    cudaFree(H->d_spins);
    cudaFree(H->d_betaf);
    cudaFree(H->d_betas);
    cudaFree(H->d_r2t);
    cudaFree(H->d_t2r);
    cudaFree(H->d_ctrl);
    cudaFree(H->d_macc);
    cudaFree(H->d_partials);
    cudaFree(H->d_obs);
    cudaFree(H->d_rec_t);
    if (H->h_stage) cudaFreeHost(H->h_stage);
    cudaFree(H->d_rec_e);
    cudaFree(H->d_rec_m);
    cudaFree(H->d_rec_h);
    if (H->own_stream) cudaStreamDestroy(H->own_stream);
    delete H;
    return ISG_OK;
}

int isg_cont_set_stream(isg_cont* H, void* stream) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_set_stream: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->stream = stream ? (cudaStream_t)stream : H->own_stream;
    return ISG_OK;
}

int isg_cont_set_temperatures(isg_cont* H, const double* temps, double J) {
    if (!H || !temps) return fail(ISG_ERR_ARG, "isg_cont_set_temperatures: NULL argument");
    cudaSetDevice(H->device);
    const int RT = H->RT;
    std::vector<double> b(RT);
    std::vector<float> bf(RT);
    for (int i = 0; i < RT; ++i) {
        if (!(temps[i] > 0.0) || !std::isfinite(temps[i]))
            return fail(ISG_ERR_ARG, "isg_cont_set_temperatures: temperatures must be positive");
        b[i] = 1.0 / temps[i];
        bf[i] = (float)b[i];
    }
    std::vector<int32_t> ident(RT);
    for (int i = 0; i < RT; ++i) ident[i] = i % H->R;
    ISG_CK(cudaMemcpyAsync(H->d_betas, b.data(), sizeof(double) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_betaf, bf.data(), sizeof(float) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->J = J;
    H->P.J = (float)J;
    H->P.Jd = J;
    H->temps_set = true;
    cont_destroy_graph(H);
    return ISG_OK;
}

int isg_cont_sweep(isg_cont* H, int64_t n_sweeps, double delta, int n_overrelax) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_sweep: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_cont_sweep: temperatures not set");
    if (n_sweeps < 0 || n_overrelax < 0 || !(delta > 0.0))
        return fail(ISG_ERR_ARG, "isg_cont_sweep: need n_sweeps >= 0, n_overrelax >= 0, delta > 0");
    cudaSetDevice(H->device);
    int64_t done = 0;
    while (done < n_sweeps) {
        const int chunk = (int)std::min<int64_t>(n_sweeps - done, 1 << 20);
        for (int j = 0; j < chunk; ++j) issue_cont_sweep(H, j, delta, n_overrelax);
        launch_cpost(H, 0, 0, 0, chunk);
        done += chunk;
    }
    return cont_check("isg_cont_sweep");
}

int isg_cont_overrelax(isg_cont* H, int colour) {
    if (!H || (colour != 0 && colour != 1))
        return fail(ISG_ERR_ARG, "isg_cont_overrelax: bad argument");
    cudaSetDevice(H->device);
    launch_or(H, colour);
    return cont_check("isg_cont_overrelax");
}

int isg_cont_metropolis(isg_cont* H, int colour, double delta) {
    if (!H || (colour != 0 && colour != 1) || !(delta > 0.0))
        return fail(ISG_ERR_ARG, "isg_cont_metropolis: bad argument");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_cont_metropolis: temperatures not set");
    cudaSetDevice(H->device);
    launch_metro(H, colour, 0, delta);
    return cont_check("isg_cont_metropolis");
}

int isg_cont_normalize(isg_cont* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_normalize: NULL handle");
    cudaSetDevice(H->device);
    k_cont_normalize<<<H->sms * 4, 256, 0, H->stream>>>(H->P, H->nc);
    return cont_check("isg_cont_normalize");
}

int isg_cont_measure(isg_cont* H, double* energy, double* mag, double* bonds) {
    if (!H || !energy || !mag) return fail(ISG_ERR_ARG, "isg_cont_measure: NULL argument");
    cudaSetDevice(H->device);
    launch_measure(H);
    int rc = cont_check("isg_cont_measure");
    if (rc) return rc;
    std::vector<double> o((size_t)H->RT * kNQ);
    ISG_CK(cudaMemcpyAsync(o.data(), H->d_obs, o.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    for (int r = 0; r < H->RT; ++r) {
        energy[r] = o[(size_t)r * kNQ];
        for (int k = 0; k < 3; ++k) mag[r * 3 + k] = o[(size_t)r * kNQ + 1 + k];
        if (bonds)
            for (int k = 0; k < 6; ++k) bonds[r * 6 + k] = o[(size_t)r * kNQ + 4 + k];
    }
    return ISG_OK;
}

int isg_cont_exchange(isg_cont* H, int parity, int64_t* accepted) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_exchange: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_cont_exchange: temperatures not set");
    cudaSetDevice(H->device);
    const int NC = H->n_classes;
    std::vector<unsigned long long> a(NC), b(NC);
    ISG_CK(cudaMemcpyAsync(a.data(), H->d_ctrl + 1 + 2 * NC, NC * 8, cudaMemcpyDeviceToHost,
                           H->stream));
    launch_cpost(H, 0, 1, parity, 0);
    int rc = cont_check("isg_cont_exchange");
    if (rc) return rc;
    ISG_CK(cudaMemcpyAsync(b.data(), H->d_ctrl + 1 + 2 * NC, NC * 8, cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    if (accepted)
        for (int s = 0; s < NC; ++s) accepted[s] = (int64_t)(b[s] - a[s]);
    return ISG_OK;
}

int isg_cont_reset_sampling(isg_cont* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_reset_sampling: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaMemsetAsync(H->d_ctrl + 1, 0, sizeof(unsigned long long) * 3 * H->n_classes,
                           H->stream));
    ISG_CK(cudaMemsetAsync(H->d_macc, 0, sizeof(unsigned long long) * H->RT, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->ksample = H->records_made = H->records_done = 0;
    return ISG_OK;
}

int isg_cont_pt_run(isg_cont* H, int64_t n_sweeps, int ee, int me, double delta, int n_or,
                    int renorm_every, int32_t* tslot, double* energy, double* mag, double* bonds,
                    int64_t max_records, int64_t* n_records) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_pt_run: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_cont_pt_run: temperatures not set");
    if (n_sweeps < 0 || ee < 1 || me < 1 || n_or < 0 || renorm_every < 0 || !(delta > 0.0))
        return fail(ISG_ERR_ARG, "isg_cont_pt_run: bad cadence or proposal arguments");
    cudaSetDevice(H->device);
    const bool keep = !tslot && !energy && !mag && !bonds;
    const uint64_t k0 = H->ksample;
    const uint64_t need = (k0 + (uint64_t)n_sweeps) / (uint64_t)me - k0 / (uint64_t)me;
    if (!keep && need > 0 && (!tslot || !energy || !mag || !bonds || max_records < (int64_t)need))
        return fail(ISG_ERR_ARG, "isg_cont_pt_run: record arrays too small");
    if (n_records) *n_records = 0;
    H->P.renorm = renorm_every;
    int64_t g = ee, b = me;
    while (b) {
        int64_t t = g % b;
        g = b;
        b = t;
    }
    const int64_t lcm = (int64_t)ee / g * me;
    const int64_t nodes = lcm * (2 * n_or + 4);
    const int period = (lcm <= 1000 && nodes <= 20000) ? (int)lcm : 0;
    const int rec_pp = period ? period / me : 0;
    const bool use_graph = period > 0 && rec_pp <= H->ring_cap / 2;
    if (H->graph && (H->g_ee != ee || H->g_me != me || H->g_nor != n_or || H->g_delta != delta ||
                     H->g_renorm != renorm_every))
        cont_destroy_graph(H);
    int64_t done = 0, row = 0;
    while (done < n_sweeps) {
        const uint64_t k = H->ksample;
        const int64_t left = n_sweeps - done;
        const uint64_t pending = H->records_made - H->records_done;
        const bool whole = use_graph && (k % (uint64_t)period) == 0 && left >= period;
        const uint64_t adds = whole ? (uint64_t)rec_pp : 1u;
        if (pending + adds > (uint64_t)H->ring_cap) {
            if (keep) {
                H->records_done = H->records_made + adds - (uint64_t)H->ring_cap;
            } else {
                int rc = cont_drain(H, tslot, energy, mag, bonds, row);
                if (rc) return rc;
                row += (int64_t)pending;
                continue;
            }
        }
        if (whole) {
            if (!H->graph) {
                cudaGraph_t gr = nullptr;
                ISG_CK(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
                for (int j = 0; j < period; ++j)
                    issue_cont_sample(H, (uint64_t)j, j, ee, me, delta, n_or,
                                      j == period - 1 ? period : 0);
                cudaError_t e = cudaStreamEndCapture(H->stream, &gr);
                if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
                e = cudaGraphInstantiate(&H->graph, gr, 0);
                cudaGraphDestroy(gr);
                if (e != cudaSuccess) {
                    H->graph = nullptr;
                    return cuda_fail(e, "cudaGraphInstantiate");
                }
                H->g_ee = ee;
                H->g_me = me;
                H->g_nor = n_or;
                H->g_delta = delta;
                H->g_renorm = renorm_every;
                H->g_period = period;
            }
            ISG_CK(cudaGraphLaunch(H->graph, H->stream));
            H->ksample += (uint64_t)period;
            H->records_made += (uint64_t)rec_pp;
            done += period;
        } else {
            const bool do_m = ((k + 1) % (uint64_t)me) == 0;
            issue_cont_sample(H, k, 0, ee, me, delta, n_or, 1);
            int rc = cont_check("isg_cont_pt_run");
            if (rc) return rc;
            H->ksample += 1;
            if (do_m) H->records_made += 1;
            done += 1;
        }
    }
    if (keep) return cont_check("isg_cont_pt_run");
    const uint64_t pending = H->records_made - H->records_done;
    int rc = cont_drain(H, tslot, energy, mag, bonds, row);
    if (rc) return rc;
    row += (int64_t)pending;
    if (n_records) *n_records = row;
    return ISG_OK;
}

int isg_cont_get_r2t(isg_cont* H, int32_t* r2t) {
    if (!H || !r2t) return fail(ISG_ERR_ARG, "isg_cont_get_r2t: NULL argument");
    cudaSetDevice(H->device);
    ISG_CK(cudaMemcpyAsync(r2t, H->d_r2t, sizeof(int32_t) * H->RT, cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

static int cont_geom(isg_cont* H, int s, int r, int64_t* n, int64_t* base, uint32_t* ps) {
    if (s < 0 || s >= H->n_classes || r < 0 || r >= H->R)
        return fail(ISG_ERR_ARG, "spin access: size index or replica out of range");
    const ContClass& C = H->P.cls[s];
    *ps = C.plane_sites;
    *n = 2 * (int64_t)C.plane_sites;
    *base = C.off + (int64_t)r * 2 * H->nc * C.plane_sites;
    return ISG_OK;
}

int isg_cont_get_spins(isg_cont* H, int s, int r, float* out) {
    if (!H || !out) return fail(ISG_ERR_ARG, "isg_cont_get_spins: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    uint32_t ps;
    int rc = cont_geom(H, s, r, &n, &base, &ps);
    if (rc) return rc;
    const int nc = H->nc;
    std::vector<float> pl((size_t)n * nc);
    ISG_CK(cudaMemcpyAsync(pl.data(), H->d_spins + base, pl.size() * sizeof(float),
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    const int L = H->sizes[s];
    for (int64_t i = 0; i < n; ++i) {
        const int64_t x = i % L, y = (i / L) % L, z = i / ((int64_t)L * L);
        const int c = (int)((x + y + z) & 1);
        for (int k = 0; k < nc; ++k)
            out[i * nc + k] = pl[(size_t)(c * nc + k) * ps + (size_t)(i >> 1)];
    }
    return ISG_OK;
}

int isg_cont_set_spins(isg_cont* H, int s, int r, const float* in) {
    if (!H || !in) return fail(ISG_ERR_ARG, "isg_cont_set_spins: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    uint32_t ps;
    int rc = cont_geom(H, s, r, &n, &base, &ps);
    if (rc) return rc;
    const int nc = H->nc;
    std::vector<float> pl((size_t)n * nc);
    const int L = H->sizes[s];
    for (int64_t i = 0; i < n; ++i) {
        const int64_t x = i % L, y = (i / L) % L, z = i / ((int64_t)L * L);
        const int c = (int)((x + y + z) & 1);
        for (int k = 0; k < nc; ++k) {
            const float v = in[i * nc + k];
            if (!std::isfinite(v)) return fail(ISG_ERR_ARG, "isg_cont_set_spins: non-finite spin");
            pl[(size_t)(c * nc + k) * ps + (size_t)(i >> 1)] = v;
        }
    }
    ISG_CK(cudaMemcpyAsync(H->d_spins + base, pl.data(), pl.size() * sizeof(float),
                           cudaMemcpyHostToDevice, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

int isg_cont_get_accepted(isg_cont* H, int64_t* accepted) {
    if (!H || !accepted) return fail(ISG_ERR_ARG, "isg_cont_get_accepted: NULL argument");
    cudaSetDevice(H->device);
    const int NC = H->n_classes;
    std::vector<unsigned long long> a(NC);
    ISG_CK(cudaMemcpyAsync(a.data(), H->d_ctrl + 1 + 2 * NC, NC * 8, cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    for (int s = 0; s < NC; ++s) accepted[s] = (int64_t)a[s];
    return ISG_OK;
}

int isg_cont_get_metro_accepted(isg_cont* H, int64_t* accepted) {
    if (!H || !accepted) return fail(ISG_ERR_ARG, "isg_cont_get_metro_accepted: NULL argument");
    cudaSetDevice(H->device);
    ISG_CK(cudaMemcpyAsync(accepted, H->d_macc, sizeof(int64_t) * H->RT, cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

int isg_cont_sync(isg_cont* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_sync: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    return cont_check("isg_cont_sync");
}

// Mean device times (ms) of one overrelaxation half-sweep, one Metropolis
// half-sweep and one measurement, on a copy that is restored afterwards.
int isg_cont_set_fused_measure(isg_cont* H, int enable) {
    if (!H) return fail(ISG_ERR_ARG, "isg_cont_set_fused_measure: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->fuse_measure = enable != 0;
    cont_destroy_graph(H);
    return ISG_OK;
}

int isg_cont_time_kernels(isg_cont* H, int n, float* out_ms) {
    if (!H || !out_ms || n < 1) return fail(ISG_ERR_ARG, "isg_cont_time_kernels: bad argument");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_cont_time_kernels: temperatures not set");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    float* backup = nullptr;
    ISG_CK(cudaMalloc((void**)&backup, sizeof(float) * (size_t)H->n_floats));
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaMemcpyAsync(backup, H->d_spins, sizeof(float) * (size_t)H->n_floats,
                                    cudaMemcpyDeviceToDevice, H->stream);
    unsigned long long ctrl0 = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&ctrl0, H->d_ctrl, sizeof(ctrl0), cudaMemcpyDeviceToHost, H->stream);
    std::vector<unsigned long long> macc(H->RT);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(macc.data(), H->d_macc, 8 * H->RT, cudaMemcpyDeviceToHost, H->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    for (int which = 0; which < 4 && e == cudaSuccess; ++which) {
        float total = 0.f;
        if (which == 3 && !H->pairs) {
            out_ms[3] = 0.f;
            break;
        }
        for (int i = 0; i < n && e == cudaSuccess; ++i) {
            e = cudaEventRecord(a, H->stream);
            if (which == 0) launch_or(H, i & 1);
            else if (which == 1) launch_metro(H, i & 1, i >> 1, 0.5);
            else if (which == 2) launch_measure(H);
            else launch_metro_measure(H, i, 0.5);
            if (e == cudaSuccess) e = cudaEventRecord(b, H->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            total += ms;
        }
        out_ms[which] = total / (float)n;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_spins, backup, sizeof(float) * (size_t)H->n_floats,
                            cudaMemcpyDeviceToDevice, H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_ctrl, &ctrl0, sizeof(ctrl0), cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_macc, macc.data(), 8 * H->RT, cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(backup);
    if (e != cudaSuccess) return cuda_fail(e, "isg_cont_time_kernels");
    return ISG_OK;
}

int isg_cont_sites_per_sweep(isg_cont* H, int64_t* sites) {
    if (!H || !sites) return fail(ISG_ERR_ARG, "isg_cont_sites_per_sweep: NULL argument");
    *sites = 2 * H->P.total_sites;
    return ISG_OK;
}

}  // extern "C"
