// isg_ising.cu — batched checkerboard Metropolis for int8 Ising spins on
// periodic cubic (dim 3) or square (dim 2) lattices, fused integer E/M
// reductions, device-side replica exchange and the PT cycle as a CUDA graph.
//
// Reference path being replaced (faulknco/ising-rs):
//   src/cuda/kernels.cu:9-56        metropolis_sweep_kernel (one launch per
//                                    replica per colour, curandState per site)
//   src/cuda/reduce_kernel.cu:7-66  reduce_mag_ising / reduce_energy_ising
//   src/cuda/lattice_gpu.rs:22-189  LatticeGpu (owner of one replica)
//   src/parallel_tempering.rs:5-36  replica_exchange (host, Xoshiro256++)
//   src/bin/gpu_fss.rs:186-286      the PT sampling loop
//
// Layout in HBM.  Every (size, replica) lattice is stored colour-split: plane
// c holds the L^dim/2 sites with (x+y+z)&1 == c at colour index
// (z*L*L + y*L + x) >> 1, so one 32-bit word carries 4 consecutive same-colour
// sites of a row.  Planes of one size are contiguous ([R][2][L^dim/2] bytes).
//
// Half-sweep kernel (one launch covers every size and replica):
//  * rolling tasks — 3D L = 32..256, a power of two: a warp walks z down a
//    column of 128 words (4 sites each), four adjacent words per lane fed
//    through a per-warp cp.async ring in shared memory; byte-parallel
//    Metropolis decisions against thresholds held as bytes.
//  * flat tasks — 3D L = 8, 16, other multiples of 8 (24, 48, 96, ...) and
//    2D: one word per lane, 32 per warp task; the x-neighbour word shifted by
//    one byte comes from the row's other lanes through __shfl_sync (or a
//    load, for rows that are not a power of two words) + funnel shift.
//  * site-block tasks — any other even L: the 16 sites of one Philox block
//    per thread, strided over the whole launch.
// All produce identical bits for the same state (the random stream is
// defined per site, not per thread).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    return ISG_ERR_CUDA;
}

constexpr int kMaxClasses = 16;
constexpr int kMaxReplicas = 1024;

// Task kinds of a lattice size (words of 4 same-colour sites of one colour
// plane of one replica):
//   kRolling (dim 3, L = 32..256): a warp task is the rows of one y-block at
//     one z, 4 adjacent words per lane (128 words; 2 and 64 if so set);
//     consecutive tasks of a size walk z, so a warp keeps the z-1, z, z+1
//     words of the other colour in registers.
//   kFlat    (other power-of-two L with L/8 dividing 32, and any other L that
//     is a multiple of 8 with whole 32-word tasks per plane, e.g. 3D L = 24,
//     48, 96, 512): 32 consecutive words, one per lane; the x-neighbour word
//     comes by shuffle from the row's lanes, or (rows that are not a power of
//     two words long) by a load.
//   kSite    (any other even L): one thread per Philox block of 16 sites
//     (site-block tasks of the same launch).
enum { kSite = 0, kFlat = 1, kRolling = 2 };

struct IsingClass {
    int L;
    int R;
    int kind;
    int log2L;
    int log2_rw;              // rw = L/8 words per row
    int log2_tpp;             // log2(tasks per plane)
    uint32_t plane_sites;     // L^dim / 2
    uint32_t tasks_per_plane; // plane_sites / 128 for word kinds
    int rep_base;             // global replica index of replica 0 (also slot base)
    int64_t spin_off;         // byte offset of replica 0 colour 0
    int64_t task_base;        // word kinds: first warp task
    int64_t task_end;
    int64_t ctask_base;       // word kinds: first CTA task (8 warp tasks); rolling
    int64_t ctask_end;        //   kinds count in work units (see log2_unit)
    int log2_groups;          // rolling: log2(column groups of 8 per replica)
    int log2_wpl;             // rolling: log2(words per lane), 1 or 2
    int log2_unit;            // rolling: a CTA task is 1 << log2_unit work units of 512 words
    int log2_rpc;             // rolling: replicas per CTA task (plane of fewer than 8 y-blocks)
    FastDiv div_half, div_L;  // site kind: divisions by L/2 and L
    FastDiv div_plane;        // site kind: division by plane_sites (when R * plane_sites < 2^31)
    int plane_fast;
    int64_t site_base;        // site kind: first site (over colour planes)
    int64_t site_end;
    // site kind, site-block tasks (site_block): S = sites of a colour per slab,
    // s_nv = v range ((L + 3) / 4 quads of S), s_nb = blocks per colour plane
    uint32_t s_nv, s_nb;
    FastDiv div_slab, div_nb;
    int sblk_fast;            // R * s_nb < 2^31: replica by multiply-high
    // flat kind with word rows that are not a power of two (L % 8 == 0):
    // indices by multiply-high, the x-neighbour word loaded, not shuffled
    int flat_gen;
    FastDiv div_rw;
    // flat kinds: a warp takes a group of up to FG consecutive tasks of a plane
    // (FG: the kernel's group size, layout_flat)
    uint32_t gpp;             // groups per plane: ceil(tasks_per_plane / 4)
    int gpp_fast;             // R * gpp < 2^31: replica by multiply-high
    FastDiv div_gpp;
    int64_t sblk_base;        // first site block of the class over all classes
    int64_t sblk_end;
};

struct IsingParams {
    uint8_t* spins;                 // down bits: 1 for s = -1, 0 for s = +1
    const uint32_t* thr;            // [slots][16]
    const uint32_t* thr8;           // [slots][4]: the thresholds as coarse bytes
    const int32_t* r2t;             // [replicas]
    unsigned long long* acc;        // [replicas][2] bond, mag
    const unsigned long long* ctrl; // ctrl[0] = global sweep base
    uint64_t seed;
    int n_classes;
    int dim;
    int64_t total_tasks;
    int64_t total_ctasks;     // rolling work units (contiguous ranges per block)
    int64_t flat_ctasks;      // flat CTA tasks (round-robin over blocks)
    int64_t total_sites;
    int64_t total_sblocks;    // site-block tasks of all site kinds
    int l2_ahead;             // rolling: planes ahead of z prefetched (0: off)
    int pf_level;             // 1: into L1, 2: into L2
    uint32_t rk0[10], rk1[10];      // Philox round keys (constant-bank operands)
    IsingClass cls[kMaxClasses];
};

// ---------------------------------------------------------------- kernels

// Loads issued where they are written (volatile asm keeps the compiler from
// sinking a prefetch next to its use).
__device__ __forceinline__ uint32_t ldg_nc(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t ldg_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint32_t pin(uint32_t x) {
    asm volatile("mov.b32 %0, %0;" : "+r"(x));
    return x;
}

// Prefetch of the 128-byte line holding p into L1 or L2 (no register result).
__device__ __forceinline__ void prefetch_line(const void* p, bool l1) {
    if (l1)
        asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
    else
        asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ uint32_t lds_u8(uint32_t saddr) {
    uint32_t v;
    asm volatile("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(saddr) : "memory");
    return v;
}
__device__ __forceinline__ void sts_u8(uint32_t saddr, uint32_t v) {
    asm volatile("st.shared.u8 [%0], %1;" ::"r"(saddr), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t lds_u32(uint32_t saddr) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(saddr));
    return v;
}

__device__ __forceinline__ uint2 lds_v2(uint32_t saddr) {
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(saddr));
    return v;
}

// Per-warp threshold table in shared memory: the 16 uint32 thresholds of the
// warp's current replica, entry own_down*8 + n_down (read by fine decisions).
__device__ __forceinline__ void load_table(uint32_t* tab, const IsingParams& P, int slot,
                                           int lane) {
    __syncwarp();
    if (lane < 16) tab[lane] = P.thr[slot * 16 + lane];
    __syncwarp();
}

// The same thresholds as bytes for the coarse decision, byte own_down*8 +
// n_down of {t0,t1,t2,t3}: 0x80 for threshold 0xFFFFFFFF (always accept), else
// threshold >> 25.
struct Thr8 {
    uint32_t t0, t1, t2, t3;
};
__device__ __forceinline__ Thr8 load_thr8(const IsingParams& P, int slot) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(P.thr8) + slot);
    return Thr8{v.x, v.y, v.z, v.w};
}

// Coarse Metropolis decision of a word of 4 same-colour sites, byte-parallel.
// ow: own down bits (bytes 0/1); nd: down-neighbour counts (bytes 0..6);
// U: the word's Philox word, byte j holding site j's coarse random in its low
// 7 bits (bit 7 ignored).  Per byte, with T the threshold byte of (own, nd),
// D = T + (0x7F - c): bit 7 is set iff c < T (the coarse random decides
// acceptance), and D == 0x7F iff c == T (a tie, decided by the fine bits).
// No byte carries into the next (T <= 0x80, c <= 0x7F).  Returns the flip mask
// (0x01 per accepted byte) and D.
__device__ __forceinline__ uint32_t coarse_flips(uint32_t ow, uint32_t nd, uint32_t U,
                                                 const Thr8& T, uint32_t& D) {
    const uint32_t sel = __byte_perm(nd | (nd >> 4), 0u, 0x0020u);  // nibbles n_down
    const uint32_t lo = __byte_perm(T.t0, T.t1, sel);                // own up
    const uint32_t hi = __byte_perm(T.t2, T.t3, sel);                // own down
    const uint32_t m = ow * 0xFFu;
    D = ((lo & ~m) | (hi & m)) + (~U & 0x7F7F7F7Fu);
    return (D >> 7) & 0x01010101u;
}
// Any tie in the word (some byte of D equal to 0x7F).
__device__ __forceinline__ bool any_tie(uint32_t D) {
    const uint32_t x = D ^ 0x7F7F7F7Fu;
    return ((x - 0x01010101u) & ~x & 0x80808080u) != 0u;
}
// Exactly the tied bytes: 0x80 in each byte of D equal to 0x7F.
__device__ __forceinline__ uint32_t tie_bytes(uint32_t D) {
    const uint32_t x = D ^ 0x7F7F7F7Fu;
    return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x | 0x7F7F7F7Fu);
}
// Fine decision of the tied sites (0x80 per byte of tmask) of word w: idx
// holds own_down*8 + n_down per byte, tab the replica's thresholds.  A tied
// site flips iff the top 25 bits of word j of the fine block 0x80000000 | w are
// <= the low 25 bits of its threshold (the top 7 are the coarse random).
__device__ __forceinline__ uint32_t fine_flips(uint32_t tmask, uint32_t idx, const uint32_t* tab,
                                               const PhiloxPre& pre, const IsingParams& P,
                                               uint32_t w) {
    const U4 f = philox_w(pre, P, 0x80000000u | w);
    const uint32_t fw[4] = {f.x, f.y, f.z, f.w};
    uint32_t flip = 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (tmask & (0x80u << (8 * j))) {
            const uint32_t t = tab[(idx >> (8 * j)) & 15u];
            if ((fw[j] >> 7) <= (t & 0x1FFFFFFu)) flip |= 1u << (8 * j);
        }
    return flip;
}

__device__ __forceinline__ void flush_acc(unsigned long long* acc, int rep, long long b,
                                          long long m, int lane) {
    // per-lane partial sums fit in int32 before the reduction
    const int sb = __reduce_add_sync(ISG_FULL_MASK, (int)b);
    const int sm = __reduce_add_sync(ISG_FULL_MASK, (int)m);
    if (lane == 0) {
        atomicAdd(&acc[2 * rep], (unsigned long long)(long long)sb);
        atomicAdd(&acc[2 * rep + 1], (unsigned long long)(long long)sm);
    }
}

// Per-lane measurement sums of the down-bit words, converted at flush time:
// bond = 4Z*n - 2Z*So - 2*Snd + 4*Sond, mag = 8*n - 2*(So + Sa).
struct MeasAcc {
    int n, so, snd, sond, sa;
};
__device__ __forceinline__ void meas_add(MeasAcc& m, uint32_t nw, uint32_t nd, uint32_t wa) {
    m.n += 1;
    m.so = __dp4a(nw, 0x01010101u, (unsigned)m.so);
    m.snd = __dp4a(nd, 0x01010101u, (unsigned)m.snd);
    m.sond = __dp4a(nw, nd, (unsigned)m.sond);
    m.sa = __dp4a(wa, 0x01010101u, (unsigned)m.sa);
}
__device__ __forceinline__ void meas_flush(unsigned long long* acc, int rep, MeasAcc& m, int Z,
                                           int lane) {
    const long long b = 4ll * Z * m.n - 2ll * Z * m.so - 2ll * m.snd + 4ll * m.sond;
    const long long g = 8ll * m.n - 2ll * (m.so + m.sa);
    flush_acc(acc, rep, b, g, lane);
    m = MeasAcc{0, 0, 0, 0, 0};
}

__device__ __forceinline__ uint2 ldg_nc2(const uint32_t* p) {
    uint2 v;
    asm volatile("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ldg_u2(const uint32_t* p) {
    uint2 v;
    asm volatile("ld.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}
__device__ __forceinline__ uint4 ldg_nc4(const uint32_t* p) {
    uint4 v;
    asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}
__device__ __forceinline__ uint4 ldg_u4(const uint32_t* p) {
    uint4 v;
    asm volatile("ld.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// Ties of the rolling half-sweep are resolved later in the same launch, 32 at
// a time: a tied site keeps its spin provisionally and its word joins the
// warp's queue {word index, per byte: own_down*8 + n_down | 0x10 if tied}.
// The fine decision only depends on the site's own spin, its neighbours of the
// other colour (unchanged during the half-sweep) and its own random bits, so
// deferring it leaves every result bit as the immediate decision would.
constexpr uint32_t kTieQ = 256;  // entries per warp (at most 31 + 128 pending)

struct TieQueue {
    uint32_t head, tail;  // warp-uniform
};

// Resolve `count` (1..32) queued entries from head: lane l takes entry
// head + l, draws its fine block, flips the accepted sites of the word in
// place (atomic XOR: the word was stored by another lane of the warp) and
// corrects the measurement sums of the provisional state.
template <int MODE>
__device__ __forceinline__ void resolve_ties(const uint2* q, uint32_t head, uint32_t count,
                                             int lane, const uint32_t* tab, const PhiloxPre& pre,
                                             const IsingParams& P, uint32_t* own, MeasAcc& macc) {
    __syncwarp();
    if ((uint32_t)lane < count) {
        const uint2 e = q[(head + (uint32_t)lane) & (kTieQ - 1)];
        const uint32_t idx = e.y & 0x0F0F0F0Fu;
        const uint32_t flip = fine_flips((e.y & 0x10101010u) << 3, idx, tab, pre, P, e.x);
        if (flip) {
            atomicXor(own + e.x, flip);
            if (MODE == 1) {
                // flipped sites leave their provisional state: down bit o -> o^1
                const uint32_t od = (idx >> 3) & flip, ou = flip & ~od;
                const uint32_t nd = idx & 0x07070707u;
                macc.so += (int)__dp4a(ou, 0x01010101u, 0u) - (int)__dp4a(od, 0x01010101u, 0u);
                macc.sond += (int)__dp4a(ou, nd, 0u) - (int)__dp4a(od, nd, 0u);
            }
        }
    }
    __syncwarp();
}

template <int MODE>
__device__ __forceinline__ void drain_ties(const uint2* q, TieQueue& tq, int lane,
                                           const uint32_t* tab, const PhiloxPre& pre,
                                           const IsingParams& P, uint32_t* own, MeasAcc& macc) {
    while (tq.tail != tq.head) {
        const uint32_t c = min(tq.tail - tq.head, 32u);
        resolve_ties<MODE>(q, tq.head, c, lane, tab, pre, P, own, macc);
        tq.head += c;
    }
}

// One z-step of a rolling column at plane offset `o` (words).  A lane owns two
// adjacent words (x, y) of a row: their new own words from the other colour's
// word pairs at z-1, z, z+1 (zm, za, zp) and the halo pair h0 (row y-1 on the
// first row of the task, y+1 on the last), with the loads of plane z+PF (own,
// halo) and z+PF+1 (other colour) issued first; PF = 2 keeps one more pair of
// each in flight (q*).  Ua / Ub: the Philox words (word z & 3 of the z quad's
// blocks) of the two words.  x neighbours: with px = (y + z + colour) & 1 the
// other colour's bytes at x - 1 + px are bytes {1,2,3} of a word + byte 0 of
// the next word (px = 1), or byte 3 of the previous word + bytes {0,1,2}
// (px = 0); one of the two is the lane's own other word, the other comes by
// one shuffle from the neighbour lane of the row (src_x, whose px is the same).
template <int MODE, int PF>
__device__ __forceinline__ void rolling_pair_step(
    const IsingParams& P, const PhiloxPre& pre, const Thr8& T8, uint32_t Ua, uint32_t Ub,
    const uint32_t* oc, const uint32_t* oa, uint32_t* mc, uint32_t col, uint32_t pz,
    uint32_t pwm, bool first, bool last, int src_up, int src_dn, int src_x, bool px,
    uint32_t sel_x, uint32_t& o, uint2& zm, uint2& za, uint2& zp, uint2& qzp, uint2& h0,
    uint2& qh0, uint2& ow, uint2& qow, MeasAcc& macc, const uint32_t* pfb, uint32_t pfo,
    bool pf_lane, uint2* q, TieQueue& tq, int lane, const uint32_t* tab, uint32_t* own) {
    const uint32_t o1 = (o + pz) & pwm, o2 = (o + 2 * pz) & pwm;
    // lanes 0..5 pull the lines of plane z + l2_ahead the warp will load
    if (pf_lane) prefetch_line(pfb + ((o + pfo) & pwm), P.pf_level == 1);
    uint2 n_zp, n_h0, n_ow;
    if constexpr (PF == 1) {
        n_zp = ldg_nc2(oc + o2);
        n_h0 = ldg_nc2(oa + o1);
        n_ow = ldg_u2(mc + o1);
    } else {
        const uint32_t o3 = (o + 3 * pz) & pwm;
        n_zp = ldg_nc2(oc + o3);
        n_h0 = ldg_nc2(oa + o2);
        n_ow = ldg_u2(mc + o2);
    }
    const uint32_t upx = __shfl_sync(ISG_FULL_MASK, za.x, src_up);
    const uint32_t upy = __shfl_sync(ISG_FULL_MASK, za.y, src_up);
    const uint32_t dnx = __shfl_sync(ISG_FULL_MASK, za.x, src_dn);
    const uint32_t dny = __shfl_sync(ISG_FULL_MASK, za.y, src_dn);
    const uint32_t nb = __shfl_sync(ISG_FULL_MASK, px ? za.x : za.y, src_x);
    const uint32_t wx0 = __byte_perm(za.x, px ? za.y : nb, sel_x);
    const uint32_t wx1 = __byte_perm(za.y, px ? nb : za.x, sel_x);
    const uint32_t nd0 = (wx0 + za.x + (last ? h0.x : upx)) + ((first ? h0.x : dnx) + zp.x + zm.x);
    const uint32_t nd1 = (wx1 + za.y + (last ? h0.y : upy)) + ((first ? h0.y : dny) + zp.y + zm.y);
    uint2 nw = ow;
    if (MODE != 2) {
        uint32_t d0, d1;
        nw.x = ow.x ^ coarse_flips(ow.x, nd0, Ua, T8, d0);
        nw.y = ow.y ^ coarse_flips(ow.y, nd1, Ub, T8, d1);
        *reinterpret_cast<uint2*>(mc + o) = nw;
        const bool t0 = any_tie(d0), t1 = any_tie(d1);
        if (__any_sync(ISG_FULL_MASK, t0 || t1)) {
            const uint32_t b0 = __ballot_sync(ISG_FULL_MASK, t0);
            const uint32_t b1 = __ballot_sync(ISG_FULL_MASK, t1);
            const uint32_t lt = (1u << lane) - 1u;
            if (t0)
                q[(tq.tail + __popc(b0 & lt)) & (kTieQ - 1)] =
                    make_uint2(o + col, (nd0 + (ow.x << 3)) | (tie_bytes(d0) >> 3));
            tq.tail += __popc(b0);
            if (t1)
                q[(tq.tail + __popc(b1 & lt)) & (kTieQ - 1)] =
                    make_uint2(o + col + 1, (nd1 + (ow.y << 3)) | (tie_bytes(d1) >> 3));
            tq.tail += __popc(b1);
            while (tq.tail - tq.head >= 32u) {
                resolve_ties<MODE>(q, tq.head, 32u, lane, tab, pre, P, own, macc);
                tq.head += 32u;
            }
        }
    }
    if (MODE != 0) {
        meas_add(macc, nw.x, nd0, za.x);
        meas_add(macc, nw.y, nd1, za.y);
    }
    zm = za;
    za = zp;
    if constexpr (PF == 1) {
        zp = n_zp;
        h0 = n_h0;
        ow = n_ow;
    } else {
        zp = qzp;
        qzp = n_zp;
        h0 = qh0;
        qh0 = n_h0;
        ow = qow;
        qow = n_ow;
    }
    o = o1;
}

// Tie queue of the four-words-per-lane path: one entry per lane-step with a
// tie in any of its four words, holding the raw per-word values the fine
// decision needs, so that appending costs no per-word selection: the first
// word index, per word own_down*8 + n_down per byte, and the coarse values D
// (tied bytes are those equal to 0x7F).  A step appends at most 32 entries
// and 32 are resolved whenever that many are pending, so at most 63 wait.
constexpr uint32_t kQuadQ = 64;
struct QuadTies {
    uint32_t w[kQuadQ];
    uint4 idx[kQuadQ];
    uint4 d[kQuadQ];
};

// Byte-wise zero test of D ^ 0x7F7F7F7F without the final mask: OR the
// values of several words, then (acc & 0x80808080) != 0 iff some byte of
// some word is a tie (exact for this any-test).
__device__ __forceinline__ uint32_t tie_acc(uint32_t D) {
    const uint32_t x = D ^ 0x7F7F7F7Fu;
    return (x - 0x01010101u) & ~x;
}

// Resolve `count` (1..32) queued lane-step entries from head: lane l takes
// entry head + l and decides each of its tied words in turn (one fine block
// per tied word; lanes with more tied words take more turns).
template <int MODE>
__device__ __forceinline__ void resolve_quad(const QuadTies& Q, uint32_t head, uint32_t count,
                                             int lane, const uint32_t* tab, const PhiloxPre& pre,
                                             const IsingParams& P, uint32_t* own, MeasAcc& macc) {
    __syncwarp();
    if ((uint32_t)lane < count) {
        const uint32_t s = (head + (uint32_t)lane) & (kQuadQ - 1);
        const uint32_t w0 = Q.w[s];
        const uint4 I = Q.idx[s], D = Q.d[s];
        const uint32_t t0 = tie_bytes(D.x), t1 = tie_bytes(D.y), t2 = tie_bytes(D.z),
                       t3 = tie_bytes(D.w);
        uint32_t tm = (t0 ? 1u : 0u) | (t1 ? 2u : 0u) | (t2 ? 4u : 0u) | (t3 ? 8u : 0u);
        while (tm) {
            const uint32_t k = (uint32_t)(__ffs(tm) - 1);
            tm &= tm - 1u;
            const bool k1 = (k & 1u) != 0, k2 = (k & 2u) != 0;
            const uint32_t tb = k2 ? (k1 ? t3 : t2) : (k1 ? t1 : t0);
            const uint32_t idx = k2 ? (k1 ? I.w : I.z) : (k1 ? I.y : I.x);
            const uint32_t flip = fine_flips(tb, idx, tab, pre, P, w0 + k);
            if (flip) {
                atomicXor(own + w0 + k, flip);
                if (MODE == 1) {
                    const uint32_t od = (idx >> 3) & flip, ou = flip & ~od;
                    const uint32_t nd = idx & 0x07070707u;
                    macc.so += (int)__dp4a(ou, 0x01010101u, 0u) - (int)__dp4a(od, 0x01010101u, 0u);
                    macc.sond += (int)__dp4a(ou, nd, 0u) - (int)__dp4a(od, nd, 0u);
                }
            }
        }
    }
    __syncwarp();
}

template <int MODE>
__device__ __forceinline__ void drain_quad(const QuadTies& Q, TieQueue& tq, int lane,
                                           const uint32_t* tab, const PhiloxPre& pre,
                                           const IsingParams& P, uint32_t* own, MeasAcc& macc) {
    while (tq.tail != tq.head) {
        const uint32_t c = min(tq.tail - tq.head, 32u);
        resolve_quad<MODE>(Q, tq.head, c, lane, tab, pre, P, own, macc);
        tq.head += c;
    }
}

// One z-step of a rolling column with four adjacent words per lane (L >=
// 32): as rolling_pair_step, with 128-bit loads and stores.  U0..U3: the
// Philox words of the four word columns for this plane.  x neighbours: the
// lane's words k-1 / k+1 and, at the row edge of the lane, word 0 of the next
// lane (px = 1) or word 3 of the previous lane (px = 0) by one shuffle.
template <int MODE, int PF>
__device__ __forceinline__ void rolling_quad_step(
    const IsingParams& P, const PhiloxPre& pre, const Thr8& T8, uint32_t U0, uint32_t U1,
    uint32_t U2, uint32_t U3, const uint32_t* oc, const uint32_t* oa, uint32_t* mc, uint32_t col,
    uint32_t pz, uint32_t pwm, bool first, bool last, int src_up, int src_dn, int src_x, bool px,
    uint32_t sel_x, uint32_t& o, uint4& zm, uint4& za, uint4& zp, uint4& qzp, uint4& h0,
    uint4& qh0, uint4& ow, uint4& qow, MeasAcc& macc, const uint32_t* pfb, uint32_t pfo,
    bool pf_lane, QuadTies& Q, TieQueue& tq, int lane, const uint32_t* tab, uint32_t* own,
    uint4* yb, uint32_t y_own, uint32_t y_halo, uint32_t y_halo_step, bool has_halo) {
    const uint32_t o1 = (o + pz) & pwm, o2 = (o + 2 * pz) & pwm;
    if (pf_lane) prefetch_line(pfb + ((o + pfo) & pwm), P.pf_level == 1);
    uint4 n_zp, n_h0, n_ow;
    if constexpr (PF == 1) {
        n_zp = ldg_nc4(oc + o2);
        n_h0 = ldg_nc4(oa + o1);
        n_ow = ldg_u4(mc + o1);
    } else {
        const uint32_t o3 = (o + 3 * pz) & pwm;
        n_zp = ldg_nc4(oc + o3);
        n_h0 = ldg_nc4(oa + o2);
        n_ow = ldg_u4(mc + o2);
    }
    // y neighbours through the warp's row buffer in shared memory: rows
    // 1..nr hold the task's rows of the other colour, row 0 the halo row
    // below the first (written by the first row's lanes), row nr + 1 the one
    // above the last; a lane reads the rows above and below its own
    __syncwarp();
    yb[y_own] = za;
    if (has_halo) yb[y_halo] = h0;
    __syncwarp();
    const uint4 yu = yb[y_own + y_halo_step], yd = yb[y_own - y_halo_step];
    const uint32_t nb = __shfl_sync(ISG_FULL_MASK, px ? za.x : za.w, src_x);
    // px = 1: bytes {1,2,3} of word k + byte 0 of word k+1; px = 0: byte 3 of
    // word k-1 + bytes {0,1,2} of word k (selects, px differs between rows)
    uint4 wx;
    wx.x = __byte_perm(za.x, px ? za.y : nb, sel_x);
    wx.y = __byte_perm(za.y, px ? za.z : za.x, sel_x);
    wx.z = __byte_perm(za.z, px ? za.w : za.y, sel_x);
    wx.w = __byte_perm(za.w, px ? nb : za.z, sel_x);
    const uint32_t nd0 = (wx.x + za.x + yu.x) + (yd.x + zp.x + zm.x);
    const uint32_t nd1 = (wx.y + za.y + yu.y) + (yd.y + zp.y + zm.y);
    const uint32_t nd2 = (wx.z + za.z + yu.z) + (yd.z + zp.z + zm.z);
    const uint32_t nd3 = (wx.w + za.w + yu.w) + (yd.w + zp.w + zm.w);
    uint4 nw = ow;
    if (MODE != 2) {
        uint32_t d0, d1, d2, d3;
        nw.x = ow.x ^ coarse_flips(ow.x, nd0, U0, T8, d0);
        nw.y = ow.y ^ coarse_flips(ow.y, nd1, U1, T8, d1);
        nw.z = ow.z ^ coarse_flips(ow.z, nd2, U2, T8, d2);
        nw.w = ow.w ^ coarse_flips(ow.w, nd3, U3, T8, d3);
        *reinterpret_cast<uint4*>(mc + o) = nw;
        const bool has =
            ((tie_acc(d0) | tie_acc(d1) | tie_acc(d2) | tie_acc(d3)) & 0x80808080u) != 0u;
        const uint32_t b = __ballot_sync(ISG_FULL_MASK, has);
        if (b != 0u) {
            // one entry per lane-step with a tie, at its rank among this
            // step's entries
            if (has) {
                const uint32_t s =
                    (tq.tail + __popc(b & ((1u << lane) - 1u))) & (kQuadQ - 1);
                Q.w[s] = o + col;
                Q.idx[s] = make_uint4(nd0 + (ow.x << 3), nd1 + (ow.y << 3), nd2 + (ow.z << 3),
                                      nd3 + (ow.w << 3));
                Q.d[s] = make_uint4(d0, d1, d2, d3);
            }
            tq.tail += __popc(b);
            if (tq.tail - tq.head >= 32u) {
                resolve_quad<MODE>(Q, tq.head, 32u, lane, tab, pre, P, own, macc);
                tq.head += 32u;
            }
        }
    }
    if (MODE != 0) {
        meas_add(macc, nw.x, nd0, za.x);
        meas_add(macc, nw.y, nd1, za.y);
        meas_add(macc, nw.z, nd2, za.z);
        meas_add(macc, nw.w, nd3, za.w);
    }
    zm = za;
    za = zp;
    if constexpr (PF == 1) {
        zp = n_zp;
        h0 = n_h0;
        ow = n_ow;
    } else {
        zp = qzp;
        qzp = n_zp;
        h0 = qh0;
        qh0 = n_h0;
        ow = qow;
        qow = n_ow;
    }
    o = o1;
}


// Four words per lane fed through a per-warp ring in shared memory (PF = 3):
// each step copies, with cp.async (straight into shared memory, no
// registers held while the copy is in flight), the lane's own words two
// planes ahead and its other-colour words (plus the halo rows) three planes
// ahead.  A ring stage of the other colour holds the task's rows at one
// plane with the halo rows below and above (row r at slots (r + 1) * lpr +
// k2), so the y neighbours are read from the stage directly.  Both rings
// have 4 stages, so with z quads aligned to z = 0 mod 4 a step's stage
// indices are compile-time constants.  Copies of a step form one group
// (empty past the end of the task): at the top of step z one group may be
// outstanding, so the one of step z - 2 (own plane z, other plane z + 1)
// is complete.
constexpr uint32_t kRingSO = 48;  // other-colour slots per stage ((nr + 2) lpr <= 48 for L <= 256)
constexpr uint32_t kRingWarpBytes = 4u * (kRingSO + 32u) * 16u;
constexpr uint32_t kRingBytes = 8u * kRingWarpBytes;  // per 256-thread block

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* g) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ uint4 lds_v4(uint32_t saddr) {
    uint4 v;
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(saddr)
                 : "memory");
    return v;
}

// Ring addresses of one warp: oth = stage 0 of the other colour, own = stage
// 0 of the own colour; y_own / y_halo: the lane's slot and its halo slot.
struct Ring {
    uint32_t oth, own, y_own, y_halo, lpr;
    bool has_halo;
};

// Copies of plane j's own words (stage j & 3) and plane j + 1's other-colour
// words (stage (j + 1) & 3) at plane offsets oj / oj1, then the group commit.
template <int SJ>
__device__ __forceinline__ void ring_issue(const Ring& G, const uint32_t* oc, const uint32_t* oa,
                                           const uint32_t* mc, uint32_t oj, uint32_t oj1,
                                           bool copy, int lane) {
    if (copy) {
        cp_async16(G.own + ((uint32_t)(SJ & 3) * 32u + (uint32_t)lane) * 16u, mc + oj);
        const uint32_t st = G.oth + (uint32_t)((SJ + 1) & 3) * kRingSO * 16u;
        cp_async16(st + G.y_own * 16u, oc + oj1);
        if (G.has_halo) cp_async16(st + G.y_halo * 16u, oa + oj1);
    }
    cp_async_commit();
}

template <int MODE, int S>
__device__ __forceinline__ void ring_quad_step(
    const IsingParams& P, const PhiloxPre& pre, const Thr8& T8, uint32_t U0, uint32_t U1,
    uint32_t U2, uint32_t U3, const Ring& G, const uint32_t* oc, const uint32_t* oa, uint32_t* mc,
    uint32_t col, uint32_t pz, uint32_t pwm, uint32_t z, uint32_t z1, int src_x, bool px,
    uint32_t sel_x, uint32_t& o, uint4& zm, uint4& za, MeasAcc& macc, const uint32_t* pfb,
    uint32_t pfo, bool pf_lane, QuadTies& Q, TieQueue& tq, int lane, const uint32_t* tab,
    uint32_t* own) {
    cp_async_wait<1>();
    __syncwarp();  // the group of step z - 2 is visible to the warp; step z - 1's reads are done
    ring_issue<S + 2>(G, oc, oa, mc, (o + 2 * pz) & pwm, (o + 3 * pz) & pwm, z + 2 < z1, lane);
    if (pf_lane) prefetch_line(pfb + ((o + pfo) & pwm), P.pf_level == 1);
    const uint32_t st = G.oth + (uint32_t)S * kRingSO * 16u;
    const uint4 zp = lds_v4(G.oth + ((uint32_t)((S + 1) & 3) * kRingSO + G.y_own) * 16u);
    const uint4 yu = lds_v4(st + (G.y_own + G.lpr) * 16u);
    const uint4 yd = lds_v4(st + (G.y_own - G.lpr) * 16u);
    const uint4 ow = lds_v4(G.own + ((uint32_t)S * 32u + (uint32_t)lane) * 16u);
    const uint32_t nb = __shfl_sync(ISG_FULL_MASK, px ? za.x : za.w, src_x);
    uint4 wx;
    wx.x = __byte_perm(za.x, px ? za.y : nb, sel_x);
    wx.y = __byte_perm(za.y, px ? za.z : za.x, sel_x);
    wx.z = __byte_perm(za.z, px ? za.w : za.y, sel_x);
    wx.w = __byte_perm(za.w, px ? nb : za.z, sel_x);
    const uint32_t nd0 = (wx.x + za.x + yu.x) + (yd.x + zp.x + zm.x);
    const uint32_t nd1 = (wx.y + za.y + yu.y) + (yd.y + zp.y + zm.y);
    const uint32_t nd2 = (wx.z + za.z + yu.z) + (yd.z + zp.z + zm.z);
    const uint32_t nd3 = (wx.w + za.w + yu.w) + (yd.w + zp.w + zm.w);
    uint4 nw = ow;
    if (MODE != 2) {
        uint32_t d0, d1, d2, d3;
        nw.x = ow.x ^ coarse_flips(ow.x, nd0, U0, T8, d0);
        nw.y = ow.y ^ coarse_flips(ow.y, nd1, U1, T8, d1);
        nw.z = ow.z ^ coarse_flips(ow.z, nd2, U2, T8, d2);
        nw.w = ow.w ^ coarse_flips(ow.w, nd3, U3, T8, d3);
        *reinterpret_cast<uint4*>(mc + o) = nw;
        const bool has =
            ((tie_acc(d0) | tie_acc(d1) | tie_acc(d2) | tie_acc(d3)) & 0x80808080u) != 0u;
        const uint32_t b = __ballot_sync(ISG_FULL_MASK, has);
        if (b != 0u) {
            if (has) {
                const uint32_t s =
                    (tq.tail + __popc(b & ((1u << lane) - 1u))) & (kQuadQ - 1);
                Q.w[s] = o + col;
                Q.idx[s] = make_uint4(nd0 + (ow.x << 3), nd1 + (ow.y << 3), nd2 + (ow.z << 3),
                                      nd3 + (ow.w << 3));
                Q.d[s] = make_uint4(d0, d1, d2, d3);
            }
            tq.tail += __popc(b);
            if (tq.tail - tq.head >= 32u) {
                resolve_quad<MODE>(Q, tq.head, 32u, lane, tab, pre, P, own, macc);
                tq.head += 32u;
            }
        }
    }
    if (MODE != 0) {
        meas_add(macc, nw.x, nd0, za.x);
        meas_add(macc, nw.y, nd1, za.y);
        meas_add(macc, nw.z, nd2, za.z);
        meas_add(macc, nw.w, nd3, za.w);
    }
    zm = za;
    za = zp;
    o = (o + pz) & pwm;
}

// Site-block tasks (any even L that is not a word size): a thread takes the
// 16 sites that share one Philox block, draws the block once and decides
// them.  The rule is the word kernels' per-site definition: with S the sites
// of a colour per slab (z-plane in 3D, row in 2D), t the slab and p the
// position in it, v = (t >> 2) S + p, the coarse random of the site is the
// low 7 bits of byte v & 3 of word t & 3 of block v >> 2, and a tie (coarse
// random equal to the threshold's top 7 bits) is decided by the top 25 bits
// of word i & 3 of the fine block 0x80000000 | (i >> 2), i = t S + p.  So
// block b holds the sites v = 4b .. 4b + 3 at the (up to) four slabs
// t = 4 (v / S) + w, w = 0..3.  Neighbours are read as bytes of the other
// colour at index z S + y L/2 + (x >> 1).
template <int DIM, int MODE>
__device__ __forceinline__ void site_block(const IsingParams& P, const IsingClass& C, int r,
                                           uint32_t b, int colour, uint32_t c2, uint32_t c3,
                                           uint32_t k0, uint32_t k1) {
    const uint32_t L = (uint32_t)C.L, half = L >> 1;
    const uint32_t S = DIM == 3 ? half * L : half;
    uint8_t* base = P.spins + C.spin_off + (int64_t)r * 2 * C.plane_sites;
    uint8_t* own = base + (int64_t)colour * C.plane_sites;
    const uint8_t* oth = base + (int64_t)(colour ^ 1) * C.plane_sites;
    const int rg = C.rep_base + r;
    const uint32_t uid = replica_uid(C.L, r);
    const uint32_t* tab = P.thr + (int64_t)(C.rep_base + (MODE != 2 ? P.r2t[rg] : 0)) * 16;
    U4 u{0u, 0u, 0u, 0u};
    if (MODE != 2) u = philox10(uid, b, c2, c3, k0, k1);
    const uint32_t W[4] = {u.x, u.y, u.z, u.w};
    int sb = 0, sm = 0;  // measurement sums of the block's sites
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t v = 4 * b + (uint32_t)j;
        if (v >= C.s_nv) break;
        const uint32_t q = fdiv(v, C.div_slab);
        const uint32_t pp = v - q * S;
        uint32_t y0 = 0, k = pp;
        if (DIM == 3) {
            y0 = fdiv(pp, C.div_half);
            k = pp - y0 * half;
        }
        // gather the (up to) four slabs' sites before deciding any
        uint32_t idx[4];
        int d[4], nd[4], oi[4];
        bool live[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t t = 4 * q + (uint32_t)w;
            live[w] = t < L;
            if (!live[w]) continue;
            const uint32_t z = DIM == 3 ? t : 0u, y = DIM == 3 ? y0 : t;
            const uint32_t x = 2 * k + ((y + z + (uint32_t)colour) & 1u);
            const uint32_t xp = x + 1 == L ? 0 : x + 1, xm = x == 0 ? L - 1 : x - 1;
            const uint32_t yp = y + 1 == L ? 0 : y + 1, ym = y == 0 ? L - 1 : y - 1;
            const uint32_t zs = z * S, row = zs + y * half;
            int n = (int)__ldg(oth + row + (xp >> 1)) + (int)__ldg(oth + row + (xm >> 1)) +
                    (int)__ldg(oth + zs + yp * half + k) + (int)__ldg(oth + zs + ym * half + k);
            if (DIM == 3) {
                const uint32_t zp = z + 1 == L ? 0 : z + 1, zm = z == 0 ? L - 1 : z - 1;
                n += (int)__ldg(oth + zp * S + y * half + k) + (int)__ldg(oth + zm * S + y * half + k);
            }
            idx[w] = row + k;
            nd[w] = n;
            d[w] = own[row + k];
            oi[w] = MODE != 0 ? (int)__ldg(oth + row + k) : 0;
        }
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            if (!live[w]) continue;
            if (MODE != 2) {
                const uint32_t th = tab[d[w] * 8 + nd[w]];
                const uint32_t c7 = (W[w] >> (8 * j)) & 0x7Fu;
                bool acc = c7 < (th >> 25);
                if (c7 == (th >> 25)) {
                    const U4 f = philox10(uid, 0x80000000u | (idx[w] >> 2), c2, c3, k0, k1);
                    const uint32_t ji = idx[w] & 3u;
                    const uint32_t fw = ji == 0 ? f.x : ji == 1 ? f.y : ji == 2 ? f.z : f.w;
                    acc = ((c7 << 25) | (fw >> 7)) <= th;
                }
                if (acc) {
                    d[w] ^= 1;
                    own[idx[w]] = (uint8_t)d[w];
                }
            }
            if (MODE != 0) {
                const int sp = 1 - 2 * d[w];
                sb += sp * (2 * DIM - 2 * nd[w]);
                sm += sp + 1 - 2 * oi[w];
            }
        }
    }
    if (MODE != 0) {
        atomicAdd(&P.acc[2 * rg], (unsigned long long)(long long)sb);
        atomicAdd(&P.acc[2 * rg + 1], (unsigned long long)(long long)sm);
    }
}

// MODE 0: update; 1: update then accumulate bond/mag of the new state;
// 2: accumulate only (no update).
//
// Work is split into CTA tasks of 8 warp tasks (blocks of 256 threads).  For
// rolling sizes the 8 warps of a CTA walk 8 adjacent y-block columns through
// the same z range, so the halo rows a warp needs are the edge rows its
// neighbours load at the same time (L1 hits); consecutive CTA tasks walk z, so
// the z-1/z/z+1 words of the other colour stay in registers (64 words per warp
// task).  Flat sizes give each warp one 32-word task per CTA task.
// PF: rolling loads issued PF planes ahead into registers (1: 3 blocks per
// SM, 2: 2 blocks per SM with more loads in flight per warp), or 3: four
// words per lane fed through the shared-memory ring (ring_quad_step); chosen
// per batch (configure_launch, isg_ising_autotune).
// WMAX: 4 if some size runs four words per lane (that path needs more
// registers: 2 blocks per SM), else 2.  MINB: blocks per SM the registers
// are budgeted for.
template <int DIM, int MODE, int PF, int WMAX, int MINB, int FG>
__global__ void __launch_bounds__(256, MINB)
    k_ising_words(const __grid_constant__ IsingParams P, int colour, int sweep_off) {
    __shared__ uint32_t s_thr[8][16];
    // per warp: the tie queue of the two-words-per-lane path or that of the
    // four-words path (a kernel runs one of the two: every rolling size of a
    // batch has the same words per lane)
    union TieStore {
        uint2 pair[kTieQ];
        QuadTies quad;
    };
    __shared__ TieStore s_ties[8];
    // four words per lane: per warp the rows of its task plus two halo rows
    // (at most (8 + 2) rows of 4 lanes, or (4 + 2) of 8, (16 + 2) of 2, (32 + 2) of 1)
    __shared__ uint4 s_y[WMAX == 4 && PF != 3 ? 8 : 1][WMAX == 4 && PF != 3 ? 80 : 1];
    // PF = 3: the per-warp rings (kRingBytes of dynamic shared memory)
    extern __shared__ uint4 s_ring[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    // rolling ranges (in work units of 512 words: one CTA task of two words
    // per lane, half of one of four) start and end on multiples of 8 units,
    // i.e. on z = 0 mod 4 (every size's unit count is a multiple of 8), so
    // each range is whole z quads
    const int64_t G = P.total_ctasks;
    int64_t ct = ((int64_t)blockIdx.x * G / gridDim.x) & ~(int64_t)7;
    const int64_t ct_end = blockIdx.x + 1 == gridDim.x
                               ? G
                               : (((int64_t)(blockIdx.x + 1) * G / gridDim.x) & ~(int64_t)7);
    int64_t ft = blockIdx.x;  // flat CTA tasks: blockIdx.x, + gridDim.x, ...

    // Launched as a programmatic dependent of the previous kernel of the
    // stream (when enabled): everything above depends on parameters only;
    // wait here for the previous grid (and its memory) before the first read
    // of device state, then let the next kernel's blocks be scheduled as ours
    // retire.  Both are no-ops for an ordinary launch.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    const uint64_t sweep = P.ctrl[0] + (uint64_t)sweep_off;
    const uint32_t c2 = (uint32_t)sweep;
    const uint32_t c3 = counter_word3(ISG_TAG_ISING, (uint32_t)colour, sweep);
    const uint32_t* tab = s_thr[wib];
    uint2* q = s_ties[wib].pair;
    QuadTies& qq = s_ties[wib].quad;
    constexpr int Z = 2 * DIM;

    int ci = 0;
    int cur_rep = -1;
    uint32_t* cur_own = nullptr;  // own plane of cur_rep (queued ties refer to it)
    MeasAcc macc{0, 0, 0, 0, 0};
    PhiloxPre pre{};
    Thr8 T8{0u, 0u, 0u, 0u};
    TieQueue tq{0u, 0u};

    while (ct < ct_end || ft < P.flat_ctasks) {
        // flat tasks first (short, latency-bound), spread over all blocks
        const bool flat_now = ft < P.flat_ctasks;
        const int64_t key = flat_now ? ft : ct;
        ci = 0;
        while (ci < kMaxClasses - 1 &&
               (P.cls[ci].kind != (flat_now ? kFlat : kRolling) || P.cls[ci].ctask_end <= key))
            ++ci;
        const IsingClass& C = P.cls[ci];
        const int64_t lct = flat_now ? key - C.ctask_base : (key - C.ctask_base) >> C.log2_unit;
        const uint32_t L = (uint32_t)C.L, Lm = L - 1;
        const int lrw = C.log2_rw;
        const uint32_t rw = 1u << lrw, rwm = rw - 1;
        const uint32_t k4 = (uint32_t)lane & rwm;
        const int src_prev = lane - (int)k4 + (int)((k4 - 1) & rwm);
        const int src_next = lane - (int)k4 + (int)((k4 + 1) & rwm);
        int r;
        uint32_t z0 = 0, z1 = 0, yb = 0;
        int64_t wt = 0;
        if (DIM == 3 && !flat_now) {
            // CTA task -> (replica group, column group g, z), z fastest; warp
            // wib takes y-block (g << lc) + (wib mod 2^lc) of replica
            // group * rpc + (wib >> lc), lc = log2(y-blocks per CTA task)
            const int lg = C.log2_groups + C.log2L;
            const int lc = 3 - C.log2_rpc;
            r = (int)(lct >> lg) * (1 << C.log2_rpc) + (wib >> lc);
            const uint32_t rem = (uint32_t)(lct & (((int64_t)1 << lg) - 1));
            z0 = rem & Lm;
            yb = ((rem >> C.log2L) << lc) + ((uint32_t)wib & ((1u << lc) - 1));
            const int64_t zlim = (int64_t)z0 + ((ct_end - ct) >> C.log2_unit);
            z1 = (uint32_t)(zlim < (int64_t)L ? zlim : (int64_t)L);
            ct += (int64_t)(z1 - z0) << C.log2_unit;
            if (r >= C.R) continue;  // the last replica group may be short
        } else {
            // flat: warp task (FG = 1) or group of up to FG tasks 8*lct + wib
            // of this size
            wt = (lct << 3) + wib;
            ft += gridDim.x;
            if constexpr (FG == 1) {
                if (wt >= C.task_end - C.task_base) continue;
                r = (int)(wt >> C.log2_tpp);
            } else {
                if (wt >= (int64_t)C.gpp * C.R) continue;
                r = C.gpp_fast ? (int)fdiv((uint32_t)wt, C.div_gpp) : (int)(wt / (int64_t)C.gpp);
            }
        }
        const int rg = C.rep_base + r;
        uint8_t* base = P.spins + C.spin_off + (int64_t)r * 2 * C.plane_sites;
        uint32_t* own = reinterpret_cast<uint32_t*>(base + (int64_t)colour * C.plane_sites);
        const uint32_t* oth =
            reinterpret_cast<const uint32_t*>(base + (int64_t)(colour ^ 1) * C.plane_sites);
        if (rg != cur_rep) {
            if (MODE != 2) {
                if (WMAX == 4)
                    drain_quad<MODE>(qq, tq, lane, tab, pre, P, cur_own, macc);
                else
                    drain_ties<MODE>(q, tq, lane, tab, pre, P, cur_own, macc);
            }
            if (MODE != 0 && cur_rep >= 0) meas_flush(P.acc, cur_rep, macc, Z, lane);
            cur_rep = rg;
            cur_own = own;
            if (MODE != 2) {
                const int slot = C.rep_base + P.r2t[rg];
                load_table(s_thr[wib], P, slot, lane);
                T8 = load_thr8(P, slot);
                pre = philox_pre(replica_uid(C.L, r), c2, c3, P.rk0[0], P.rk1[0]);
            }
        }

        if (DIM == 3 && !flat_now) {
            // a warp task: 32 * wpl words (nr rows of rw words), wpl = 2 or 4
            // adjacent words per lane; a row has 1 (L = 32) to 16 lanes and a
            // task 2 to 32 rows; when the task is the whole plane (L = 32),
            // the y shuffles wrap around it and the halo rows are its own
            const int lw = C.log2_wpl;
            const uint32_t pz = L << lrw;          // words per z-plane
            const uint32_t pwm = (pz << C.log2L) - 1;  // plane words - 1 (power of two)
            const int lh = lrw - lw;               // log2(lanes per row)
            const uint32_t k2 = (uint32_t)lane & ((1u << lh) - 1);
            const uint32_t col = (yb << (5 + lw)) + ((uint32_t)lane << lw);  // the lane's first word
            const uint32_t rb = (uint32_t)lane >> lh, nr = 32u >> lh;
            const uint32_t y = yb * nr + rb;
            const bool first = rb == 0, last = rb == nr - 1;
            const uint32_t ha = (((first ? y - 1 : y + 1) & Lm) << lrw) | (k2 << lw);
            const int src_up = (lane + (1 << lh)) & 31, src_dn = (lane - (1 << lh)) & 31;
            const uint32_t km = (1u << lh) - 1;
            const int src_prev2 = lane - (int)k2 + (int)((k2 - 1) & km);
            const int src_next2 = lane - (int)k2 + (int)((k2 + 1) & km);
            const uint32_t* oc = oth + col;   // column base pointers
            const uint32_t* oa = oth + ha;
            uint32_t* mc = own + col;
            // cache prefetch: lanes [0, n) the n = 2^lw 128-byte lines of the
            // task's own words, [n, 2n) those of the other colour, 2n and
            // 2n + 1 the lines of the other colour's halo rows
            const int nlines = 1 << lw;
            const bool pf_lane = P.l2_ahead > 0 && lane < 2 * nlines + 2;
            const uint32_t y0 = yb * nr;
            const uint32_t* pfb =
                lane < 2 * nlines
                    ? (lane < nlines ? (const uint32_t*)own : oth) + (yb << (5 + lw)) +
                          32u * (uint32_t)(lane & (nlines - 1))
                    : oth + ((((lane == 2 * nlines ? y0 - 1 : y0 + nr) & Lm) << lrw) & ~31u);
            const uint32_t pfo = (uint32_t)P.l2_ahead * pz;
            // x-neighbour parity at even z (z0 is even) and at odd z
            const bool pe = ((y + (uint32_t)colour) & 1u) != 0;
            const int src_lo = pe ? src_next2 : src_prev2, src_hi = pe ? src_prev2 : src_next2;
            const uint32_t sel_lo = pe ? 0x4321u : 0x2107u, sel_hi = pe ? 0x2107u : 0x4321u;
            uint32_t o = z0 * pz;                        // offset of plane z
            if constexpr (WMAX == 4 && PF == 3) {
                // (a kernel with WMAX = 4 runs every rolling size at four
                // words per lane: lw == 2) ring slots: own row rb + 1; halo
                // row 0 (first row) or nr + 1 (last row); a row is lpr lanes
                const uint32_t lpr = 1u << lh;
                Ring G;
                G.oth = (uint32_t)__cvta_generic_to_shared(s_ring) + (uint32_t)wib * kRingWarpBytes;
                G.own = G.oth + 4u * kRingSO * 16u;
                G.y_own = (rb + 1) * lpr + k2;
                G.y_halo = (first ? 0u : (nr + 1) * lpr) + k2;
                G.lpr = lpr;
                G.has_halo = first || last;
                __syncwarp();  // the warp's reads of the ring in its previous task are done
                // prologue (z0 = 0 mod 4): the task's rows of the other colour
                // at z0 join the group of (own z0, other z0 + 1); then the
                // group of (own z0 + 1, other z0 + 2)
                cp_async16(G.oth + G.y_own * 16u, oc + o);
                if (G.has_halo) cp_async16(G.oth + G.y_halo * 16u, oa + o);
                ring_issue<0>(G, oc, oa, mc, o, (o + pz) & pwm, true, lane);
                ring_issue<1>(G, oc, oa, mc, (o + pz) & pwm, (o + 2 * pz) & pwm, true, lane);
                uint4 zm = ldg_nc4(oc + ((o - pz) & pwm));
                uint4 za = ldg_nc4(oc + o);
                for (uint32_t z = z0; z < z1; z += 4) {
                    U4 u0{}, u1{}, u2{}, u3{};
                    if (MODE != 2) {
                        u0 = philox_w(pre, P, (o >> 2) + col);
                        u1 = philox_w(pre, P, (o >> 2) + col + 1);
                        u2 = philox_w(pre, P, (o >> 2) + col + 2);
                        u3 = philox_w(pre, P, (o >> 2) + col + 3);
                    }
#define ISG_RING4(S, W, SRC, PX, SEL)                                                           \
    ring_quad_step<MODE, S>(P, pre, T8, u0.W, u1.W, u2.W, u3.W, G, oc, oa, mc, col, pz, pwm,     \
                            z + S, z1, SRC, PX, SEL, o, zm, za, macc, pfb, pfo, pf_lane, qq, tq, \
                            lane, tab, own)
                    ISG_RING4(0, x, src_lo, pe, sel_lo);
                    ISG_RING4(1, y, src_hi, !pe, sel_hi);
                    ISG_RING4(2, z, src_lo, pe, sel_lo);
                    ISG_RING4(3, w, src_hi, !pe, sel_hi);
#undef ISG_RING4
                }
            } else if constexpr (WMAX == 4) {
                // row buffer slots: own row rb + 1; halo row 0 (first row) or
                // nr + 1 (last row); a row is lpr lanes
                const uint32_t lpr = 1u << lh;
                const uint32_t y_own = (rb + 1) * lpr + k2;
                const uint32_t y_halo = (first ? 0u : (nr + 1) * lpr) + k2;
                uint4 zm = ldg_nc4(oc + ((o - pz) & pwm));
                uint4 za = ldg_nc4(oc + o);
                uint4 zp = ldg_nc4(oc + ((o + pz) & pwm));
                uint4 h0 = ldg_nc4(oa + o);
                uint4 ow = ldg_u4(mc + o);
                uint4 qzp{0u, 0u, 0u, 0u}, qh0{0u, 0u, 0u, 0u}, qow{0u, 0u, 0u, 0u};
                if constexpr (PF == 2) {
                    qzp = ldg_nc4(oc + ((o + 2 * pz) & pwm));
                    qh0 = ldg_nc4(oa + ((o + pz) & pwm));
                    qow = ldg_u4(mc + ((o + pz) & pwm));
                }
                // z quads (4k .. 4k+3) share one Philox block per word column:
                // counter (z>>2)*pz + word, Philox word z & 3 for plane z; the
                // four blocks of a quad are drawn together (independent chains)
                for (uint32_t z = z0; z < z1; z += 4) {
                    U4 u0{}, u1{}, u2{}, u3{};
                    if (MODE != 2) {
                        u0 = philox_w(pre, P, (o >> 2) + col);
                        u1 = philox_w(pre, P, (o >> 2) + col + 1);
                        u2 = philox_w(pre, P, (o >> 2) + col + 2);
                        u3 = philox_w(pre, P, (o >> 2) + col + 3);
                    }
#define ISG_ROLL4(W, SRC, PX, SEL)                                                            \
    rolling_quad_step<MODE, PF>(P, pre, T8, u0.W, u1.W, u2.W, u3.W, oc, oa, mc, col, pz, pwm,  \
                                first, last, src_up, src_dn, SRC, PX, SEL, o, zm, za, zp, qzp, \
                                h0, qh0, ow, qow, macc, pfb, pfo, pf_lane, qq, tq, lane, tab,  \
                                own, s_y[wib], y_own, y_halo, lpr, first || last)
                    ISG_ROLL4(x, src_lo, pe, sel_lo);
                    ISG_ROLL4(y, src_hi, !pe, sel_hi);
                    ISG_ROLL4(z, src_lo, pe, sel_lo);
                    ISG_ROLL4(w, src_hi, !pe, sel_hi);
#undef ISG_ROLL4
                }
            } else {
                uint2 zm = ldg_nc2(oc + ((o - pz) & pwm));
                uint2 za = ldg_nc2(oc + o);
                uint2 zp = ldg_nc2(oc + ((o + pz) & pwm));
                uint2 h0 = ldg_nc2(oa + o);
                uint2 ow = ldg_u2(mc + o);
                uint2 qzp{0u, 0u}, qh0{0u, 0u}, qow{0u, 0u};
                if constexpr (PF == 2) {
                    qzp = ldg_nc2(oc + ((o + 2 * pz) & pwm));
                    qh0 = ldg_nc2(oa + ((o + pz) & pwm));
                    qow = ldg_u2(mc + ((o + pz) & pwm));
                }
                for (uint32_t z = z0; z < z1; z += 4) {
                    U4 ua{}, ub{};
                    if (MODE != 2) {
                        ua = philox_w(pre, P, (o >> 2) + col);
                        ub = philox_w(pre, P, (o >> 2) + col + 1);
                    }
#define ISG_ROLL_STEP(UA, UB, SRC, PX, SEL)                                                    \
    rolling_pair_step<MODE, PF>(P, pre, T8, UA, UB, oc, oa, mc, col, pz, pwm, first, last,   \
                                src_up, src_dn, SRC, PX, SEL, o, zm, za, zp, qzp, h0, qh0, ow, \
                                qow, macc, pfb, pfo, pf_lane, q, tq, lane, tab, own)
                    ISG_ROLL_STEP(ua.x, ub.x, src_lo, pe, sel_lo);
                    ISG_ROLL_STEP(ua.y, ub.y, src_hi, !pe, sel_hi);
                    ISG_ROLL_STEP(ua.z, ub.z, src_lo, pe, sel_lo);
                    ISG_ROLL_STEP(ua.w, ub.w, src_hi, !pe, sel_hi);
#undef ISG_ROLL_STEP
                }
            }
        } else {
            if constexpr (FG == 1) {
                const uint32_t tl = (uint32_t)(wt & (int64_t)(C.tasks_per_plane - 1));
                const uint32_t w = (tl << 5) + (uint32_t)lane;
                const uint32_t row = w >> lrw;
                uint32_t y, z;
                if (DIM == 3) {
                    y = row & Lm;
                    z = row >> C.log2L;
                } else {
                    y = row;
                    z = 0;
                }
                const uint32_t yp = (y + 1) & Lm, ym = (y - 1) & Lm;
                uint32_t wa, wyp, wym, wzp = 0, wzm = 0;
                if (DIM == 3) {
                    const uint32_t zb = z << C.log2L;
                    wa = __ldg(oth + (((zb + y) << lrw) + k4));
                    wyp = __ldg(oth + (((zb + yp) << lrw) + k4));
                    wym = __ldg(oth + (((zb + ym) << lrw) + k4));
                    wzp = __ldg(oth + (((((z + 1) & Lm) << C.log2L) + y) << lrw) + k4);
                    wzm = __ldg(oth + (((((z - 1) & Lm) << C.log2L) + y) << lrw) + k4);
                } else {
                    wa = __ldg(oth + ((y << lrw) + k4));
                    wyp = __ldg(oth + ((yp << lrw) + k4));
                    wym = __ldg(oth + ((ym << lrw) + k4));
                }
                const uint32_t p = (y + z + (uint32_t)colour) & 1u;
                const uint32_t prev = __shfl_sync(ISG_FULL_MASK, wa, src_prev);
                const uint32_t next = __shfl_sync(ISG_FULL_MASK, wa, src_next);
                const uint32_t wx = p ? __funnelshift_r(wa, next, 8) : __funnelshift_l(prev, wa, 8);
                uint32_t nd = wx + wa + wyp + wym;
                if (DIM == 3) nd += wzp + wzm;
                const uint32_t ow = own[w];
                uint32_t nw = ow;
                if (MODE != 2) {
                    // z (3D) or y (2D) quad of this word: one Philox block, word t & 3
                    const uint32_t t = DIM == 3 ? z : y;
                    const uint32_t slab = DIM == 3 ? (L << lrw) : rw;
                    const U4 u = philox_w(pre, P, w - (t - (t >> 2)) * slab);
                    const uint32_t U = (t & 2u) ? ((t & 1u) ? u.w : u.z) : ((t & 1u) ? u.y : u.x);
                    uint32_t d;
                    nw = ow ^ coarse_flips(ow, nd, U, T8, d);
                    if (any_tie(d)) nw ^= fine_flips(tie_bytes(d), nd + (ow << 3), tab, pre, P, w);
                    own[w] = nw;
                }
                if (MODE != 0) meas_add(macc, nw, nd, wa);
            } else {
                // a flat group: up to (uint32_t)FG consecutive 32-word tasks of one plane,
                // one word per lane each; all loads of the group are issued
                // before any decision (one task at a time waits on each load)
                const uint32_t grp = (uint32_t)(wt - (int64_t)r * C.gpp);
                uint32_t fw[FG], fa[FG], fn[FG], fyp[FG], fym[FG], fzp[FG], fzm[FG], fo[FG], fy[FG], fz[FG];
    #pragma unroll
                for (int g = 0; g < FG; ++g) {
                    const uint32_t tl = grp * (uint32_t)FG + (uint32_t)g;
                    if (tl >= C.tasks_per_plane) break;  // warp-uniform
                    const uint32_t w = (tl << 5) + (uint32_t)lane;
                    uint32_t y, z;
                    fzp[g] = fzm[g] = fn[g] = 0u;
                    if (C.flat_gen) {
                        // rows of rwg = L / 8 words, not a power of two: the
                        // row's x-neighbour word (wrapping) is loaded
                        const uint32_t rwg = L >> 3;
                        const uint32_t row = fdiv(w, C.div_rw);
                        const uint32_t kk = w - row * rwg;
                        if (DIM == 3) {
                            z = fdiv(row, C.div_L);
                            y = row - z * L;
                        } else {
                            y = row;
                            z = 0;
                        }
                        const uint32_t yp = y + 1 == L ? 0 : y + 1, ym = y == 0 ? L - 1 : y - 1;
                        const uint32_t p = (y + z + (uint32_t)colour) & 1u;
                        const uint32_t kx =
                            p ? (kk + 1 == rwg ? 0 : kk + 1) : (kk == 0 ? rwg - 1 : kk - 1);
                        const uint32_t zb = z * L;
                        fa[g] = __ldg(oth + (zb + y) * rwg + kk);
                        fn[g] = __ldg(oth + (zb + y) * rwg + kx);
                        fyp[g] = __ldg(oth + (zb + yp) * rwg + kk);
                        fym[g] = __ldg(oth + (zb + ym) * rwg + kk);
                        if (DIM == 3) {
                            const uint32_t zp = z + 1 == L ? 0 : z + 1, zm = z == 0 ? L - 1 : z - 1;
                            fzp[g] = __ldg(oth + (zp * L + y) * rwg + kk);
                            fzm[g] = __ldg(oth + (zm * L + y) * rwg + kk);
                        }
                    } else {
                        const uint32_t row = w >> lrw;
                        if (DIM == 3) {
                            y = row & Lm;
                            z = row >> C.log2L;
                        } else {
                            y = row;
                            z = 0;
                        }
                        const uint32_t yp = (y + 1) & Lm, ym = (y - 1) & Lm;
                        const uint32_t zb = DIM == 3 ? z << C.log2L : 0u;
                        fa[g] = __ldg(oth + (((zb + y) << lrw) + k4));
                        fyp[g] = __ldg(oth + (((zb + yp) << lrw) + k4));
                        fym[g] = __ldg(oth + (((zb + ym) << lrw) + k4));
                        if (DIM == 3) {
                            fzp[g] = __ldg(oth + (((((z + 1) & Lm) << C.log2L) + y) << lrw) + k4);
                            fzm[g] = __ldg(oth + (((((z - 1) & Lm) << C.log2L) + y) << lrw) + k4);
                        }
                    }
                    fw[g] = w;
                    fy[g] = y;
                    fz[g] = z;
                    fo[g] = own[w];
                }
    #pragma unroll
                for (int g = 0; g < FG; ++g) {
                    if (grp * (uint32_t)FG + (uint32_t)g >= C.tasks_per_plane) break;
                    const uint32_t w = fw[g], wa = fa[g], y = fy[g], z = fz[g], ow = fo[g];
                    const uint32_t p = (y + z + (uint32_t)colour) & 1u;
                    uint32_t wx;
                    if (C.flat_gen) {
                        wx = p ? __funnelshift_r(wa, fn[g], 8) : __funnelshift_l(fn[g], wa, 8);
                    } else {
                        const uint32_t prev = __shfl_sync(ISG_FULL_MASK, wa, src_prev);
                        const uint32_t next = __shfl_sync(ISG_FULL_MASK, wa, src_next);
                        wx = p ? __funnelshift_r(wa, next, 8) : __funnelshift_l(prev, wa, 8);
                    }
                    uint32_t nd = wx + wa + fyp[g] + fym[g];
                    if (DIM == 3) nd += fzp[g] + fzm[g];
                    uint32_t nw = ow;
                    if (MODE != 2) {
                        // z (3D) or y (2D) quad of this word: one Philox block, word t & 3
                        const uint32_t t = DIM == 3 ? z : y;
                        const uint32_t slab = DIM == 3 ? L * (L >> 3) : L >> 3;  // words per slab
                        const U4 u = philox_w(pre, P, w - (t - (t >> 2)) * slab);
                        const uint32_t U = (t & 2u) ? ((t & 1u) ? u.w : u.z) : ((t & 1u) ? u.y : u.x);
                        uint32_t d;
                        nw = ow ^ coarse_flips(ow, nd, U, T8, d);
                        if (any_tie(d)) nw ^= fine_flips(tie_bytes(d), nd + (ow << 3), tab, pre, P, w);
                        own[w] = nw;
                    }
                    if (MODE != 0) meas_add(macc, nw, nd, wa);
                }
            }
        }
    }
    if (MODE != 2) {
        if (WMAX == 4)
            drain_quad<MODE>(qq, tq, lane, tab, pre, P, cur_own, macc);
        else
            drain_ties<MODE>(q, tq, lane, tab, pre, P, cur_own, macc);
    }
    if (MODE != 0 && cur_rep >= 0) meas_flush(P.acc, cur_rep, macc, Z, lane);

    // site-block tasks (even L that are not word sizes): one Philox block's
    // 16 sites per thread, strided over every thread of the launch
    if (P.total_sblocks > 0) {
        const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < P.total_sblocks;
             g += stride) {
            int sc = 0;
            while (P.cls[sc].sblk_end <= g) ++sc;
            const IsingClass& C = P.cls[sc];
            const int64_t lg = g - C.sblk_base;
            const int r = C.sblk_fast ? (int)fdiv((uint32_t)lg, C.div_nb) : (int)(lg / C.s_nb);
            const uint32_t b = (uint32_t)(lg - (int64_t)r * C.s_nb);
            site_block<DIM, MODE>(P, C, r, b, colour, c2, c3, k0, k1);
        }
    }
}

// Small lattices, whole schedules in one launch: one thread-block cluster per
// lattice (lattice l = size l / R, replica l % R).  CTA c of the cluster keeps
// colour indices [c*chunk, (c+1)*chunk) of both colour planes in its shared
// memory for the whole launch; neighbours owned by other CTAs are read through
// distributed shared memory (mapa + ld.shared::cluster), and hardware cluster
// barriers (release / acquire at cluster scope) separate the half-sweeps.
// Spins are loaded from HBM at the start and written back at the end.  Same
// per-site update rule and random stream as the site-block tasks
// (site_block), so any launch shape gives the same bits.
constexpr int kResidentThreads = 1024;

struct ResidentParams {
    const uint32_t* tables;   // [n][16] threshold tables
    const int32_t* sched;     // per-sweep table index, or null: the lattice's slot table
    unsigned long long* rec;  // [rows][lattices][2] bond, mag (zeroed before the launch)
    uint64_t sweep0;          // global sweep number of sweep 0
    int64_t n_sweeps;
    int measure_every;        // 0: no records
    int measure_phase;        // record after sweep k iff k % every == phase
    int lattices;
    int cs;                   // CTAs per lattice (the cluster size)
    int log2_chunk;           // colour indices per CTA and plane: 1 << log2_chunk
    FastDiv div_half[kMaxClasses];  // L/2
    FastDiv div_L[kMaxClasses];
    // parallel tempering (pt != 0; one site per thread): the PT cycle of
    // k_ising_post inside the launch.  Sampling sweep ks0 + k is measured when
    // (ks0 + k + 1) % me == 0 and exchanges when (ks0 + k + 1) % ee == 0; at
    // an exchange every lattice publishes its energy, all blocks meet at a
    // bounded grid barrier, and every CTA computes its size's exchange pass on
    // its own copy of the ladder (the same FP64 arithmetic as k_ising_post).
    int pt, ee, me;
    uint64_t ks0;
    int32_t* rec_t;               // [rows][lattices] slot of each record
    unsigned long long* eacc;     // [lattices][2] bond, mag of the current measurement (zeroed)
    double* ebuf;                 // [2][lattices] energies at exchange points
    int32_t* r2t;
    int32_t* t2r;
    const double* betas;          // per slot
    unsigned long long* ctrl;     // PostParams layout: [1+NC+s] exchanges, [1+2NC+s] accepted
    unsigned int* bar;            // grid barrier [arrivals, generation] (zeroed)
    int* err;                     // set when a barrier wait gives up
    double J, h;
    uint64_t seed;
    int n_classes;
};

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
                 ::: "memory");
}
__device__ __forceinline__ void cluster_arrive() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Byte j of colour plane `pl` of the cluster's lattice: owner CTA j >> lc.
__device__ __forceinline__ int dsm_spin(uint32_t sbase, uint32_t pl, uint32_t j, int lc) {
    const uint32_t local = sbase + (pl << lc) + (j & ((1u << lc) - 1u));
    uint32_t remote, v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(j >> lc));
    asm volatile("ld.shared::cluster.u8 %0, [%1];" : "=r"(v) : "r"(remote) : "memory");
    return (int)v;
}

// Neighbour colour indices, Philox block and word/half selector of the site at
// colour index i (see site_gather).
template <int DIM>
__device__ __forceinline__ void resident_geom(uint32_t i, uint32_t L, uint32_t half, uint32_t S,
                                              const FastDiv& dh, const FastDiv& dL,
                                              uint32_t colour, uint32_t (&nb)[6], uint32_t& c1,
                                              uint32_t& sel) {
    const uint32_t row = fdiv(i, dh);
    const uint32_t k = i - row * half;
    uint32_t y, z;
    if (DIM == 3) {
        z = fdiv(row, dL);
        y = row - z * L;
    } else {
        y = row;
        z = 0;
    }
    const uint32_t x = 2 * k + ((y + z + colour) & 1u);
    const uint32_t xp = x + 1 == L ? 0 : x + 1, xm = x == 0 ? L - 1 : x - 1;
    const uint32_t yp = y + 1 == L ? 0 : y + 1, ym = y == 0 ? L - 1 : y - 1;
    const uint32_t rowL = (z * L + y) * L;
    nb[0] = (rowL + xp) >> 1;
    nb[1] = (rowL + xm) >> 1;
    nb[2] = ((z * L + yp) * L + x) >> 1;
    nb[3] = ((z * L + ym) * L + x) >> 1;
    if (DIM == 3) {
        const uint32_t zp = z + 1 == L ? 0 : z + 1, zm = z == 0 ? L - 1 : z - 1;
        nb[4] = ((zp * L + y) * L + x) >> 1;
        nb[5] = ((zm * L + y) * L + x) >> 1;
    } else {
        nb[4] = nb[5] = 0;
    }
    const uint32_t t = DIM == 3 ? z : y;
    const uint32_t v = (t >> 2) * S + (i - t * S);
    c1 = v >> 2;
    sel = (v & 3u) | ((t & 3u) << 2);  // byte v & 3 of word t & 3
}

__device__ __forceinline__ uint32_t dsm_map(uint32_t local, uint32_t rank) {
    uint32_t remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(rank));
    return remote;
}
__device__ __forceinline__ int dsm_ld(uint32_t remote) {
    uint32_t v;
    asm volatile("ld.shared::cluster.u8 %0, [%1];" : "=r"(v) : "r"(remote) : "memory");
    return (int)v;
}

// Flip decision from the site's coarse block u (selector sel: byte sel & 3 of
// word sel >> 2) and, on a tie with the threshold's top 7 bits, the fine block
// of counter 0x80000000 | (i >> 2) drawn with the same hoisted rounds.
__device__ __forceinline__ bool resident_accept(const U4& u, uint32_t sel, uint32_t th,
                                                uint32_t i, const PhiloxPre& pre,
                                                const IsingParams& P) {
    const uint32_t jw = sel >> 2;
    const uint32_t uw = jw == 0 ? u.x : jw == 1 ? u.y : jw == 2 ? u.z : u.w;
    const uint32_t c7 = (uw >> (8u * (sel & 3u))) & 0x7Fu;
    bool acc = c7 < (th >> 25);
    if (c7 == (th >> 25)) {
        const U4 f = philox_w(pre, P, 0x80000000u | (i >> 2));
        const uint32_t ji = i & 3u;
        const uint32_t fw = ji == 0 ? f.x : ji == 1 ? f.y : ji == 2 ? f.z : f.w;
        acc = ((c7 << 25) | (fw >> 7)) <= th;
    }
    return acc;
}

// One half-sweep of the fast path: the thread's site (if any) of this colour,
// with its neighbour addresses, Philox index and selector fixed for the launch.
template <int DIM, int COLOUR>
__device__ __forceinline__ void resident_fast_half(
    const IsingParams& P, const uint32_t* tab, uint32_t uid, uint64_t sweep, bool has, uint32_t i,
    const uint32_t (&na)[6], uint32_t own_addr, uint32_t oth_addr, uint32_t c1, uint32_t sel,
    bool meas, int& bsum, int& msum) {
    const uint32_t c3 = counter_word3(ISG_TAG_ISING, (uint32_t)COLOUR, sweep);
    const PhiloxPre pre = philox_pre(uid, (uint32_t)sweep, c3, P.rk0[0], P.rk1[0]);
    if (!has) return;
    int nd = dsm_ld(na[0]) + dsm_ld(na[1]) + dsm_ld(na[2]) + dsm_ld(na[3]);
    if (DIM == 3) nd += dsm_ld(na[4]) + dsm_ld(na[5]);
    int d = (int)lds_u8(own_addr);
    const uint32_t th = tab[d * 8 + nd];
    const U4 u = philox_w(pre, P, c1);
    if (resident_accept(u, sel, th, i, pre, P)) {
        d ^= 1;
        sts_u8(own_addr, (uint32_t)d);
    }
    if (COLOUR == 1 && meas) {
        const int sp = 1 - 2 * d;
        bsum += sp * (2 * DIM - 2 * nd);
        msum += sp + 1 - 2 * (int)lds_u8(oth_addr);
    }
}

template <int DIM>
__device__ __forceinline__ int resident_nd(uint32_t sbase, uint32_t pl, int lc,
                                           const uint32_t (&nb)[6]) {
    int nd = dsm_spin(sbase, pl, nb[0], lc) + dsm_spin(sbase, pl, nb[1], lc) +
             dsm_spin(sbase, pl, nb[2], lc) + dsm_spin(sbase, pl, nb[3], lc);
    if (DIM == 3) nd += dsm_spin(sbase, pl, nb[4], lc) + dsm_spin(sbase, pl, nb[5], lc);
    return nd;
}

// The PT form of the resident kernel's one-site-per-thread loop (Q.pt).
template <int DIM>
__device__ __forceinline__ void resident_pt_loop(
    const IsingParams& P, const ResidentParams& Q, uint32_t* tab, int lid, int crank, int s, int r,
    int rg, uint32_t uid, bool has, uint32_t i, const uint32_t (&na0)[6],
    const uint32_t (&na1)[6], uint32_t a0, uint32_t a1, uint32_t c10, uint32_t c11,
    uint32_t sel0, uint32_t sel1) {
    __shared__ int s_t2r[kMaxReplicas], s_r2t[kMaxReplicas];
    __shared__ double s_e[kMaxReplicas];
    __shared__ int s_acc, s_ok;
    const int R = P.cls[0].R;
    const int base = s * R;
    const int lane = threadIdx.x & 31;
    const uint32_t bd = blockDim.x;
    const int NC = Q.n_classes;
    for (int j = threadIdx.x; j < R; j += bd) {
        s_t2r[j] = Q.t2r[base + j];
        s_r2t[j] = Q.r2t[base + j];
    }
    if (threadIdx.x == 0) {
        s_acc = 0;
        s_ok = 1;
    }
    unsigned long long xc = Q.ctrl[1 + NC + s];
    __syncthreads();
    const uint64_t ks0 = Q.ks0;
    const int64_t row0 = (int64_t)(ks0 / (uint64_t)Q.me);
    for (int64_t k = 0; k < Q.n_sweeps; ++k) {
        const uint64_t ks = ks0 + (uint64_t)k;
        const bool do_m = ((ks + 1) % (uint64_t)Q.me) == 0;
        const bool do_x = ((ks + 1) % (uint64_t)Q.ee) == 0;
        const bool meas = do_m || do_x;
        const uint64_t sweep = Q.sweep0 + (uint64_t)k;
        int bsum = 0, msum = 0;
        resident_fast_half<DIM, 0>(P, tab, uid, sweep, has, i, na0, a0, a1, c10, sel0, meas, bsum,
                                   msum);
        cluster_sync_all();
        resident_fast_half<DIM, 1>(P, tab, uid, sweep, has, i, na1, a1, a0, c11, sel1, meas, bsum,
                                   msum);
        if (meas) {
            bsum = __reduce_add_sync(ISG_FULL_MASK, bsum);
            msum = __reduce_add_sync(ISG_FULL_MASK, msum);
            // before the cluster barrier, so CTA 0 sees every warp's sums
            if (lane == 0 && (bsum != 0 || msum != 0)) {
                atomicAdd(&Q.eacc[2 * lid], (unsigned long long)(long long)bsum);
                atomicAdd(&Q.eacc[2 * lid + 1], (unsigned long long)(long long)msum);
            }
        }
        cluster_sync_all();
        if (!meas) continue;
        if (crank == 0 && threadIdx.x == 0) {
            const long long b = (long long)atomicExch(&Q.eacc[2 * lid], 0ull);
            const long long m = (long long)atomicExch(&Q.eacc[2 * lid + 1], 0ull);
            if (do_m) {
                const int64_t row = (int64_t)((ks + 1) / (uint64_t)Q.me) - 1 - row0;
                Q.rec[(row * Q.lattices + lid) * 2] = (unsigned long long)b;
                Q.rec[(row * Q.lattices + lid) * 2 + 1] = (unsigned long long)m;
                Q.rec_t[row * Q.lattices + lid] = s_r2t[r];
            }
            if (do_x) {
                const double t1 = __dmul_rn(Q.J, (double)b);
                const double t2 = __dmul_rn(Q.h, (double)m);
                Q.ebuf[(xc & 1ull) * Q.lattices + lid] = __dsub_rn(-t1, t2);
            }
        }
        if (!do_x) continue;
        // every lattice's energy of this exchange point, then the pass
        const bool ok = grid_barrier(Q.bar, Q.err, gridDim.x);
        // the cluster follows its CTA 0's outcome, so that all its CTAs leave
        // (or go on) at the same point; a wait that gave up set Q.err, which
        // every block sees at the next barrier at the latest
        if (threadIdx.x == 0) s_ok = ok ? 1 : 0;
        cluster_sync_all();
        uint32_t ok0 = 1;
        {
            const uint32_t local = (uint32_t)__cvta_generic_to_shared(&s_ok);
            asm volatile("ld.shared::cluster.u32 %0, [%1];"
                         : "=r"(ok0)
                         : "r"(dsm_map(local, 0u))
                         : "memory");
        }
        cluster_sync_all();
        if (!ok0) {
            if (threadIdx.x == 0) s_ok = 0;
            __syncthreads();
            break;
        }
        for (int j = threadIdx.x; j < R; j += bd)
            s_e[j] = __ldcg(Q.ebuf + (xc & 1ull) * Q.lattices + base + j);
        __syncthreads();
        const int par = (int)(xc & 1ull);
        const uint32_t k0 = (uint32_t)Q.seed, k1 = (uint32_t)(Q.seed >> 32);
        const uint32_t c3 = counter_word3(ISG_TAG_EXCH, 0, xc);
        for (int j = par + 2 * (int)threadIdx.x; j + 1 < R; j += 2 * (int)bd) {
            const int ri = s_t2r[j], rj = s_t2r[j + 1];
            const double d = __dmul_rn(__dsub_rn(Q.betas[base + j], Q.betas[base + j + 1]),
                                       __dsub_rn(s_e[rj], s_e[ri]));
            bool acc = d < 0.0;
            if (!acc) {
                const U4 u = philox10(exchange_uid(P.cls[s].L), (uint32_t)j, (uint32_t)xc, c3, k0, k1);
                acc = uniform53(u.x, u.y) < exp(-d);
            }
            if (acc) {
                s_t2r[j] = rj;
                s_t2r[j + 1] = ri;
                s_r2t[ri] = j + 1;
                s_r2t[rj] = j;
                atomicAdd(&s_acc, 1);
            }
        }
        ++xc;
        __syncthreads();
        // the table of this lattice's (possibly new) slot
        if (threadIdx.x < 16) tab[threadIdx.x] = Q.tables[(int64_t)(base + s_r2t[r]) * 16 + threadIdx.x];
        __syncthreads();
    }
    // the ladder, exchange count and acceptances back to the handle's state
    if (crank == 0) {
        if (threadIdx.x == 0) Q.r2t[rg] = s_r2t[r];
        if (r == 0) {
            for (int j = threadIdx.x; j < R; j += bd) Q.t2r[base + j] = s_t2r[j];
            if (threadIdx.x == 0 && s_ok) {
                Q.ctrl[1 + NC + s] = xc;
                Q.ctrl[1 + 2 * NC + s] += (unsigned long long)s_acc;
            }
        }
    }
    cluster_sync_all();
}

template <int DIM>
__global__ void __launch_bounds__(kResidentThreads, 1)
    k_ising_resident(const __grid_constant__ IsingParams P, const __grid_constant__ ResidentParams Q) {
    extern __shared__ __align__(16) uint8_t s_spin[];  // [2][chunk]
    __shared__ uint32_t s_tab[2][16];                  // tables of sweeps k and k+1
    const int lid = blockIdx.x / Q.cs;
    const int crank = blockIdx.x - lid * Q.cs;
    const int R = P.cls[0].R;
    const int s = lid / R, r = lid - s * R;
    const IsingClass& C = P.cls[s];
    const FastDiv dh = Q.div_half[s], dL = Q.div_L[s];
    const uint32_t plane = C.plane_sites, L = (uint32_t)C.L, half = L >> 1;
    const uint32_t S = plane / L;
    const int lc = Q.log2_chunk;
    const uint32_t chunk = 1u << lc;
    const uint32_t i0 = min(plane, (uint32_t)crank << lc), i1 = min(plane, i0 + chunk);
    uint8_t* base = P.spins + C.spin_off + (int64_t)r * 2 * plane;
    const uint32_t uid = replica_uid(C.L, r);
    const int rg = C.rep_base + r;
    const int lane = threadIdx.x & 31;
    const uint32_t bd = blockDim.x;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(s_spin);
    for (uint32_t j = threadIdx.x; j < i1 - i0; j += bd) {
        s_spin[j] = base[i0 + j];
        s_spin[chunk + j] = base[plane + i0 + j];
    }
    // sweep k uses s_tab[k & 1]; the table of sweep k+1 is fetched during sweep k
    if (threadIdx.x < 16) {
        const int64_t t0 = Q.sched ? (int64_t)Q.sched[0] : (int64_t)(C.rep_base + P.r2t[rg]);
        const uint32_t v = Q.tables[t0 * 16 + threadIdx.x];
        s_tab[0][threadIdx.x] = v;
        s_tab[1][threadIdx.x] = v;
    }
    cluster_sync_all();
    if (chunk <= bd) {
        // at most one site per thread and colour: addresses fixed for the launch
        const uint32_t i = i0 + threadIdx.x;
        const bool has = i < i1;
        constexpr int NB = 2 * DIM;
        uint32_t na0[6] = {0, 0, 0, 0, 0, 0}, na1[6] = {0, 0, 0, 0, 0, 0};
        uint32_t c10 = 0, c11 = 0, sel0 = 0, sel1 = 0;
        if (has) {
            uint32_t nb[6];
            resident_geom<DIM>(i, L, half, S, dh, dL, 0u, nb, c10, sel0);
#pragma unroll
            for (int j = 0; j < NB; ++j)
                na0[j] = dsm_map(sbase + chunk + (nb[j] & (chunk - 1u)), nb[j] >> lc);
            resident_geom<DIM>(i, L, half, S, dh, dL, 1u, nb, c11, sel1);
#pragma unroll
            for (int j = 0; j < NB; ++j)
                na1[j] = dsm_map(sbase + (nb[j] & (chunk - 1u)), nb[j] >> lc);
        }
        const uint32_t a0 = sbase + (i - i0), a1 = sbase + chunk + (i - i0);
        if (Q.pt) {
            resident_pt_loop<DIM>(P, Q, s_tab[0], lid, crank, s, r, rg, uid, has, i, na0, na1, a0,
                                  a1, c10, c11, sel0, sel1);
        } else
        for (int64_t k = 0; k < Q.n_sweeps; ++k) {
            const uint32_t* tab = s_tab[k & 1];
            uint32_t tnext = 0;
            const bool fetch = Q.sched && threadIdx.x < 16 && k + 1 < Q.n_sweeps;
            if (fetch) tnext = Q.tables[(int64_t)Q.sched[k + 1] * 16 + threadIdx.x];
            const uint64_t sweep = Q.sweep0 + (uint64_t)k;
            const bool meas = Q.measure_every > 0 && (k % Q.measure_every) == Q.measure_phase;
            int bsum = 0, msum = 0;
            resident_fast_half<DIM, 0>(P, tab, uid, sweep, has, i, na0, a0, a1, c10, sel0, meas,
                                       bsum, msum);
            cluster_sync_all();
            resident_fast_half<DIM, 1>(P, tab, uid, sweep, has, i, na1, a1, a0, c11, sel1, meas,
                                       bsum, msum);
            if (fetch) s_tab[(k + 1) & 1][threadIdx.x] = tnext;
            if (meas) {
                bsum = __reduce_add_sync(ISG_FULL_MASK, bsum);
                msum = __reduce_add_sync(ISG_FULL_MASK, msum);
            }
            cluster_arrive();
            if (meas && lane == 0 && (bsum != 0 || msum != 0)) {
                const int64_t row = k / Q.measure_every;
                unsigned long long* rp = Q.rec + (row * Q.lattices + lid) * 2;
                atomicAdd(rp, (unsigned long long)(long long)bsum);
                atomicAdd(rp + 1, (unsigned long long)(long long)msum);
            }
            cluster_wait();
        }
    } else {
    for (int64_t k = 0; k < Q.n_sweeps; ++k) {
        const uint32_t* tab = s_tab[k & 1];
        uint32_t tnext = 0;
        const bool fetch = Q.sched && threadIdx.x < 16 && k + 1 < Q.n_sweeps;
        if (fetch) tnext = Q.tables[(int64_t)Q.sched[k + 1] * 16 + threadIdx.x];
        const uint64_t sweep = Q.sweep0 + (uint64_t)k;
        const bool meas = Q.measure_every > 0 && (k % Q.measure_every) == Q.measure_phase;
#pragma unroll 1
        for (uint32_t colour = 0; colour < 2; ++colour) {
            const uint32_t c2 = (uint32_t)sweep;
            const uint32_t c3 = counter_word3(ISG_TAG_ISING, colour, sweep);
            uint8_t* own = s_spin + (colour << lc) - i0;  // own[i] for i in [i0, i1)
            const uint32_t oc = colour ^ 1u;
            const bool mc = colour == 1 && meas;
            int bsum = 0, msum = 0;
            const PhiloxPre pre = philox_pre(uid, c2, c3, P.rk0[0], P.rk1[0]);
#pragma unroll 1
            for (uint32_t i = i0 + threadIdx.x; i < i1; i += bd) {
                uint32_t nb[6], c1, sel;
                resident_geom<DIM>(i, L, half, S, dh, dL, colour, nb, c1, sel);
                const int nd = resident_nd<DIM>(sbase, oc, lc, nb);
                int d = own[i];
                const uint32_t th = tab[d * 8 + nd];
                const U4 u = philox_w(pre, P, c1);
                if (resident_accept(u, sel, th, i, pre, P)) {
                    d ^= 1;
                    own[i] = (uint8_t)d;
                }
                if (mc) {
                    const int sp = 1 - 2 * d;
                    bsum += sp * (2 * DIM - 2 * nd);
                    msum += sp + 1 - 2 * (int)s_spin[(oc << lc) + (i - i0)];
                }
            }
            if (colour == 1 && fetch) s_tab[(k + 1) & 1][threadIdx.x] = tnext;
            if (mc) {
                bsum = __reduce_add_sync(ISG_FULL_MASK, bsum);
                msum = __reduce_add_sync(ISG_FULL_MASK, msum);
            }
            // the record atomics go out between arrive and wait: the release
            // orders the shared-memory spins, the atomics overlap the barrier
            cluster_arrive();
            if (mc && lane == 0 && (bsum != 0 || msum != 0)) {
                const int64_t row = k / Q.measure_every;
                unsigned long long* rp = Q.rec + (row * Q.lattices + lid) * 2;
                atomicAdd(rp, (unsigned long long)(long long)bsum);
                atomicAdd(rp + 1, (unsigned long long)(long long)msum);
            }
            cluster_wait();
        }
    }
    }
    for (uint32_t j = threadIdx.x; j < i1 - i0; j += bd) {
        base[i0 + j] = s_spin[j];
        base[plane + i0 + j] = s_spin[chunk + j];
    }
}

// Hot start: natural site n of replica r gets -1 if the top bit of word
// (n & 3) of Philox(uid, n >> 2, 0, INIT) is set, else +1 (stored as the
// down bit).
__global__ void k_ising_init(const __grid_constant__ IsingParams P, int dim) {
    const uint32_t k0 = (uint32_t)P.seed, k1 = (uint32_t)(P.seed >> 32);
    const uint32_t c3 = counter_word3(ISG_TAG_INIT, 0, 0);
    for (int ci = 0; ci < P.n_classes; ++ci) {
        const IsingClass& C = P.cls[ci];
        const int64_t nsite = 2 * (int64_t)C.plane_sites;
        const int64_t total = nsite * C.R;
        for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total;
             g += (int64_t)gridDim.x * blockDim.x) {
            const int r = (int)(g / nsite);
            const uint32_t n = (uint32_t)(g - (int64_t)r * nsite);
            const U4 u = philox10(replica_uid(C.L, r), n >> 2, 0, c3, k0, k1);
            const uint32_t j = n & 3u;
            const uint32_t wv = j == 0 ? u.x : j == 1 ? u.y : j == 2 ? u.z : u.w;
            const uint32_t L = (uint32_t)C.L;
            const uint32_t x = n % L;
            const uint32_t y = (n / L) % L;
            const uint32_t z = dim == 3 ? n / (L * L) : 0;
            const uint32_t c = (x + y + z) & 1u;
            P.spins[C.spin_off + (int64_t)r * nsite + (int64_t)c * C.plane_sites + (n >> 1)] =
                (uint8_t)(wv >> 31);
        }
    }
}

struct PostParams {
    unsigned long long* acc;  // [replicas][2]
    int32_t* r2t;
    int32_t* t2r;
    const double* betas;      // per slot
    int32_t* rec_t;
    long long* rec_b;
    long long* rec_m;
    unsigned long long* ctrl; // [0] sweep base, [1+s] records, [1+NC+s] xcount, [1+2NC+s] accepted
    long long ring_cap;
    double J, h;
    uint64_t seed;
    int R;
    int n_classes;
    int replicas_total;
    int L[kMaxClasses];
    // energy histograms (NULL when off): per size s and slot t, bins b of the
    // bond sum B = 4 b - dN_s (B + dN is a multiple of 4 on a periodic even
    // lattice), 4 counters per bin: samples, and the sums of |m|, m^2, m^4 in
    // units of 2^-32; hist_rng[2 (s R + t) + {0, 1}] = lowest / highest bin seen
    unsigned long long* hist;
    int32_t* hist_rng;
    long long hist_off[kMaxClasses];   // first bin of size s
    long long hist_dn[kMaxClasses];    // dim * N_s
    double hist_nsite[kMaxClasses];    // N_s
};

// One block per size: record (slot, bond, mag) of every replica, run an
// exchange pass, zero the accumulators, advance the sweep counter.
// Exchange arithmetic follows src/parallel_tempering.rs:17-33 in FP64 with
// explicitly rounded products so the CPU replay matches bit for bit.
__global__ void k_ising_post(const __grid_constant__ PostParams Q, int do_record, int do_exchange,
                             int parity, int zero_acc, int advance) {
    __shared__ double s_e[kMaxReplicas];
    __shared__ int s_t2r[kMaxReplicas];
    __shared__ int s_acc;
    const int s = blockIdx.x;
    const int R = Q.R;
    const int base = s * R;
    const int NC = Q.n_classes;
    unsigned long long* rec_count = Q.ctrl + 1 + s;
    unsigned long long* xcount = Q.ctrl + 1 + NC + s;
    unsigned long long* accepted = Q.ctrl + 1 + 2 * NC + s;
    if (threadIdx.x == 0) s_acc = 0;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const long long b = (long long)Q.acc[2 * (base + r)];
        const long long m = (long long)Q.acc[2 * (base + r) + 1];
        const double t1 = __dmul_rn(Q.J, (double)b);
        const double t2 = __dmul_rn(Q.h, (double)m);
        s_e[r] = __dsub_rn(-t1, t2);
        s_t2r[r] = Q.t2r[base + r];
        if (do_record) {
            const long long slot = (long long)(*rec_count % (unsigned long long)Q.ring_cap);
            const long long o = slot * Q.replicas_total + base + r;
            const int t = Q.r2t[base + r];
            Q.rec_t[o] = t;
            Q.rec_b[o] = b;
            Q.rec_m[o] = m;
            if (Q.hist) {
                // one replica per slot, so no two threads share a bin row
                const long long dn = Q.hist_dn[s];
                const long long bin = (b + dn) >> 2;
                unsigned long long* hb =
                    Q.hist + 4 * (Q.hist_off[s] + (long long)t * ((dn >> 1) + 1) + bin);
                const double m1 = __ddiv_rn(fabs((double)m), Q.hist_nsite[s]);
                const double m2 = __dmul_rn(m1, m1);
                const double m4 = __dmul_rn(m2, m2);
                hb[0] += 1ull;
                hb[1] += __double2ull_rn(__dmul_rn(m1, 4294967296.0));
                hb[2] += __double2ull_rn(__dmul_rn(m2, 4294967296.0));
                hb[3] += __double2ull_rn(__dmul_rn(m4, 4294967296.0));
                int32_t* rg = Q.hist_rng + 2 * (base + t);
                rg[0] = min(rg[0], (int32_t)bin);
                rg[1] = max(rg[1], (int32_t)bin);
            }
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
    if (zero_acc)
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            Q.acc[2 * (base + r)] = 0ull;
            Q.acc[2 * (base + r) + 1] = 0ull;
        }
    if (threadIdx.x == 0) {
        if (do_record) *rec_count += 1ull;
        if (s == 0 && advance) Q.ctrl[0] += (unsigned long long)advance;
    }
}

// Natural-layout +-1 bytes <-> colour-split down-bit planes of one replica.
__global__ void k_ising_nat_to_planes(uint8_t* __restrict__ planes, const int8_t* __restrict__ nat,
                                      int L, int dim, uint32_t half) {
    const uint32_t n = 2 * half;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % (uint32_t)L, y = (i / (uint32_t)L) % (uint32_t)L;
        const uint32_t z = dim == 3 ? i / ((uint32_t)L * (uint32_t)L) : 0;
        const uint32_t c = (x + y + z) & 1u;
        planes[c * half + (i >> 1)] = nat[i] < 0 ? 1 : 0;
    }
}
__global__ void k_ising_planes_to_nat(const uint8_t* __restrict__ planes, int8_t* __restrict__ nat,
                                      int L, int dim, uint32_t half) {
    const uint32_t n = 2 * half;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % (uint32_t)L, y = (i / (uint32_t)L) % (uint32_t)L;
        const uint32_t z = dim == 3 ? i / ((uint32_t)L * (uint32_t)L) : 0;
        const uint32_t c = (x + y + z) & 1u;
        nat[i] = planes[c * half + (i >> 1)] ? (int8_t)-1 : (int8_t)1;
    }
}

// ---------------------------------------------------------------- host object

static int num_sms(int dev) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

static int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace isg

using namespace isg;

struct isg_ising {
    int device = 0;
    int dim = 3;
    int n_classes = 0;
    int R = 0;
    int replicas_total = 0;
    uint64_t seed = 0;
    std::vector<int> sizes;
    IsingParams P{};
    PostParams Q{};
    uint8_t* d_spins = nullptr;
    int64_t spin_bytes = 0;
    uint32_t* d_thr = nullptr;
    uint32_t* d_thr8 = nullptr;
    int32_t* d_r2t = nullptr;
    int32_t* d_t2r = nullptr;
    double* d_betas = nullptr;
    unsigned long long* d_acc = nullptr;
    unsigned long long* d_ctrl = nullptr;
    int64_t ring_cap = 0;
    unsigned char* h_stage = nullptr;  // pinned staging of drained records (kStageRows rows)
    int32_t* d_rec_t = nullptr;
    long long* d_rec_b = nullptr;
    long long* d_rec_m = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    bool temps_set = false;
    double J = 1.0, h = 0.0;
    int threads = 256;
    int blocks_per_sm = 0;
    int prefetch = 0;          // rolling prefetch depth as set (0: automatic)
    int wpl_max = 4;           // rolling words per lane for L >= 128 (2 or 4)
    int wmax = 2;              // word kernel variant: 4 if some size runs 4 words per lane
    int flatg = 1;             // flat tasks per warp group (layout_flat)
    bool cache_pf_set = false; // cache prefetch set by the caller (else automatic)
    bool pdl = true;           // word kernels as programmatic dependent launches
    int pf = 1;                // depth in use
    int word_grid = 0;
    int word_grids[3] = {1, 1, 1};
    int sms = 1;
    // sampling-phase mirror of the device counters
    uint64_t ksample = 0;
    uint64_t records_done = 0;  // records already copied out of the ring
    uint64_t records_made = 0;
    uint64_t gsweep = 0;
    // cached cycle graph
    cudaGraphExec_t graph = nullptr;
    int graph_ee = 0, graph_me = 0, graph_period = 0;
    // cached graph of kStepGraphSweeps plain sweeps (isg_ising_step)
    cudaGraphExec_t step_graph = nullptr;
    // schedule buffers (isg_ising_run_schedule)
    uint32_t* d_sched_tab = nullptr;
    int64_t sched_tab_cap = 0;
    int32_t* d_sched = nullptr;
    int64_t sched_cap = 0;
    unsigned long long* d_srec = nullptr;
    int64_t srec_cap = 0;
    // resident PT (small lattices): record slots and exchange scratch
    bool resident_pt = true;
    int32_t* d_srec_t = nullptr;
    int64_t srec_t_cap = 0;
    unsigned long long* d_pt_scratch = nullptr;  // eacc [RT][2], ebuf [2][RT], bar, err
    int64_t pt_scratch_cap = 0;
    // energy histograms (isg_ising_hist_*)
    unsigned long long* d_hist = nullptr;
    int32_t* d_hist_rng = nullptr;
    int64_t hist_bins = 0;  // all sizes and slots
};

namespace isg {

// CTA tasks of the rolling sizes: warp tasks of 32 * wpl words (wpl = 2 for
// L = 64, else wpl_max) are the rows of one y-block at one z; 8 y-blocks of
// a plane form a column group, and a CTA task is one (replica, group, z), z
// fastest, so consecutive CTA tasks walk z.
static void layout_rolling(isg_ising* H) {
    IsingParams& P = H->P;
    int64_t ctask = 0;
    H->wmax = 2;
    for (int s = 0; s < H->n_classes; ++s) {
        IsingClass& C = P.cls[s];
        if (C.kind != kRolling) continue;
        const int L = C.L, rw = L / 8;
        C.log2_wpl = H->wpl_max == 4 ? 2 : 1;
        const int tw = 32 << C.log2_wpl;          // words per warp task
        const int cols = L * rw / tw;             // y-blocks per plane
        // a CTA task is 8 y-blocks of one plane, or, when a plane has fewer
        // (four words per lane: 4 at L = 64, 1 at L = 32), the plane of
        // 8 / cols replicas
        const int groups = cols >= 8 ? cols / 8 : 1;
        const int rpc = cols >= 8 ? 1 : 8 / cols;
        C.log2_groups = 0;
        while ((1 << C.log2_groups) < groups) ++C.log2_groups;
        C.log2_rpc = 0;
        while ((1 << C.log2_rpc) < rpc) ++C.log2_rpc;
        // blocks split the rolling work by words, not by CTA tasks: a CTA
        // task of four words per lane counts twice
        C.log2_unit = C.log2_wpl - 1;
        C.ctask_base = ctask;
        ctask += ((int64_t)((C.R + rpc - 1) / rpc) * groups * L) << C.log2_unit;
        C.ctask_end = ctask;
        if (C.log2_wpl == 2) H->wmax = 4;
    }
    P.total_ctasks = ctask;
}

// CTA tasks of the flat sizes: groups of FG consecutive warp tasks of one
// plane per warp, 8 groups per CTA task.  FG = 1 (the original one-task form)
// unless some size has rows that are not a power of two words long (its
// tasks read the x-neighbour word from memory) or the flat work is large
// (at least 8192 warp tasks, e.g. 2D L = 256 x 32): several tasks in flight
// per warp then hide the latency (2D L = 256 x 128: +24%), while a batch of a
// few small lattices needs every warp it can get (3D L = 8, 16 x 128: -26%
// with groups).  FG = 4, or 2 next to four-words-per-lane rolling sizes (the
// groups' registers would cost that kernel more).
static void layout_flat(isg_ising* H) {
    IsingParams& P = H->P;
    bool gen = false;
    int64_t tasks = 0;
    for (int s = 0; s < H->n_classes; ++s)
        if (P.cls[s].kind == kFlat) {
            gen = gen || P.cls[s].flat_gen;
            tasks += (int64_t)P.cls[s].tasks_per_plane * P.cls[s].R;
        }
    H->flatg = !(gen || tasks >= 8192) ? 1 : H->wmax == 4 ? 2 : 4;
    int64_t fctask = 0;
    for (int s = 0; s < H->n_classes; ++s) {
        IsingClass& C = P.cls[s];
        if (C.kind != kFlat) continue;
        C.gpp = (C.tasks_per_plane + (uint32_t)H->flatg - 1) / (uint32_t)H->flatg;
        C.div_gpp = make_div(std::max<uint32_t>(1u, C.gpp));
        C.gpp_fast = (int64_t)C.gpp * C.R < ((int64_t)1 << 31) ? 1 : 0;
        C.ctask_base = fctask;
        fctask += ((int64_t)C.gpp * C.R + 7) / 8;
        C.ctask_end = fctask;
    }
    P.flat_ctasks = fctask;
}

template <int DIM, int PF, int WMAX, int MINB, int FG>
static void (*word_kernel_m(int mode))(IsingParams, int, int) {
    if (mode == 0) return k_ising_words<DIM, 0, PF, WMAX, MINB, FG>;
    if (mode == 1) return k_ising_words<DIM, 1, PF, WMAX, MINB, FG>;
    return k_ising_words<DIM, 2, PF, WMAX, MINB, FG>;
}

// Variants: two words per lane at 3 blocks per SM (one plane ahead) or 2
// (two planes ahead); four words per lane at 2 blocks per SM (one or two
// planes ahead; at 3 blocks per SM its registers spill and it ran 10-19%
// slower).
static void (*word_kernel(int dim, int mode, int pf, int wmax, int fg))(IsingParams, int, int) {
    if (dim == 3) {
        if (wmax == 4) {
            if (fg > 1) {
                if (pf == 3) return word_kernel_m<3, 3, 4, 2, 2>(mode);
                if (pf == 2) return word_kernel_m<3, 2, 4, 2, 2>(mode);
                return word_kernel_m<3, 1, 4, 2, 2>(mode);
            }
            if (pf == 3) return word_kernel_m<3, 3, 4, 2, 1>(mode);
            if (pf == 2) return word_kernel_m<3, 2, 4, 2, 1>(mode);
            return word_kernel_m<3, 1, 4, 2, 1>(mode);
        }
        if (fg > 1) {  // (the flat groups' registers: 2 blocks per SM)
            if (pf == 2) return word_kernel_m<3, 2, 2, 2, 4>(mode);
            return word_kernel_m<3, 1, 2, 2, 4>(mode);
        }
        if (pf == 2) return word_kernel_m<3, 2, 2, 2, 1>(mode);
        return word_kernel_m<3, 1, 2, 3, 1>(mode);
    }
    // no rolling tasks in 2D: one form per flat group size
    if (fg > 1) return word_kernel_m<2, 1, 2, 3, 4>(mode);
    return word_kernel_m<2, 1, 2, 3, 1>(mode);
}

// Dynamic shared memory of the word kernel: the per-warp rings of PF = 3.
static size_t word_smem(const isg_ising* H) {
    return H->dim == 3 && H->wmax == 4 && H->pf == 3 ? (size_t)kRingBytes : 0;
}

// Word kernels run 256-thread blocks (one CTA task = 8 warp tasks); the
// grid is SMs x blocks per SM (occupancy maximum unless set), at most one
// block per CTA task.  `threads` applies to the site kernel.  Prefetch form:
// as set, else the shared-memory ring with four words per lane (5% faster at
// L = 128 x 128 than loads one plane ahead in registers, 7% on the mixed PT
// batch), and with two words per lane 2 when the batch's spins fit in L2
// (latency of L2 hits is hidden better by loads further ahead) and 1
// otherwise (three blocks per SM keep more DRAM requests in flight) —
// measured on both kinds of workload.
static int configure_launch(isg_ising* H) {
    const int thr = H->threads;
    // one launch per half-sweep covers every size: rolling ranges, flat
    // groups and site-block tasks (256 per block)
    const int64_t need = std::max<int64_t>(std::max<int64_t>(H->P.total_ctasks, H->P.flat_ctasks),
                                           (H->P.total_sblocks + 255) / 256);
    const bool in_l2 = H->spin_bytes <= ((int64_t)96 << 20);
    // two words per lane: loads two planes ahead help L2-resident batches;
    // four words per lane (2 blocks per SM either way): one plane ahead
    H->pf = H->prefetch > 0 ? H->prefetch : (H->wmax == 4 ? 3 : in_l2 ? 2 : 1);
    if (H->dim != 3 || (H->pf == 3 && H->wmax != 4)) H->pf = H->dim == 3 && in_l2 ? 2 : 1;
    // batches larger than L2 on the register paths: lines 3 planes ahead
    // prefetched into L2 (the ring's copies run far enough ahead without)
    if (!H->cache_pf_set) {
        H->P.l2_ahead = in_l2 || H->pf == 3 ? 0 : 3;
        H->P.pf_level = 2;
    }
    const size_t dyn = word_smem(H);
    for (int mode = 0; mode < 3; ++mode) {
        int occ = 0;
        const void* fn = (const void*)word_kernel(H->dim, mode, H->pf, H->wmax, H->flatg);
        if (dyn > 0) {
            cudaError_t a =
                cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
            if (a != cudaSuccess) return cuda_fail(a, "cudaFuncSetAttribute");
        }
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 256, dyn);
        if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        if (occ < 1) occ = 1;
        const int bps = H->blocks_per_sm > 0 ? std::min(H->blocks_per_sm, occ) : occ;
        const int64_t max_blocks = (int64_t)H->sms * bps;
        H->word_grids[mode] = (int)std::max<int64_t>(1, std::min(max_blocks, need));
    }
    H->word_grid = H->word_grids[0];
    (void)thr;
    return ISG_OK;
}

static void launch_half(isg_ising* H, int colour, int sweep_off, int mode) {
    if (H->P.total_tasks > 0 || H->P.total_sites > 0) {
        // programmatic dependent launch: the word kernel's blocks may be
        // scheduled while the previous kernel drains (they wait on it first)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)H->word_grids[mode]);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = word_smem(H);
        cfg.stream = H->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = H->pdl ? 1 : 0;
        cudaLaunchKernelEx(&cfg, word_kernel(H->dim, mode, H->pf, H->wmax, H->flatg), H->P, colour,
                           sweep_off);
    }
}

static void launch_post(isg_ising* H, int do_record, int do_exchange, int parity, int zero_acc,
                        int advance) {
    int thr = std::min(1024, std::max(32, ((H->R + 31) / 32) * 32));
    k_ising_post<<<H->n_classes, thr, 0, H->stream>>>(H->Q, do_record, do_exchange, parity,
                                                      zero_acc, advance);
}

static int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return ISG_OK;
}

static void destroy_graph(isg_ising* H) {
    if (H->graph) cudaGraphExecDestroy(H->graph);
    H->graph = nullptr;
    H->graph_period = 0;
    if (H->step_graph) cudaGraphExecDestroy(H->step_graph);
    H->step_graph = nullptr;
}

// Plain sweeps (no measurement, no exchange) replayed as one graph: every
// node reads the sweep base from the device counter, so replays continue the
// random stream.
constexpr int kStepGraphSweeps = 64;

// One sampling sweep k (0-based) issued directly.
static void issue_sample_sweep(isg_ising* H, uint64_t k, int sweep_off, int ee, int me,
                               int advance) {
    const bool do_m = ((k + 1) % (uint64_t)me) == 0;
    const bool do_x = ((k + 1) % (uint64_t)ee) == 0;
    launch_half(H, 0, sweep_off, 0);
    launch_half(H, 1, sweep_off, (do_m || do_x) ? 1 : 0);
    if (do_m || do_x || advance)
        launch_post(H, do_m ? 1 : 0, do_x ? 1 : 0, -1, (do_m || do_x) ? 1 : 0, advance);
}

static int build_graph(isg_ising* H, int ee, int me, int period) {
    destroy_graph(H);
    cudaGraph_t g = nullptr;
    ISG_CK(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
    for (int j = 0; j < period; ++j)
        issue_sample_sweep(H, (uint64_t)j, j, ee, me, j == period - 1 ? period : 0);
    cudaError_t e = cudaStreamEndCapture(H->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&H->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        H->graph = nullptr;
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    H->graph_ee = ee;
    H->graph_me = me;
    H->graph_period = period;
    return ISG_OK;
}

// Records leave the device ring through a pinned staging buffer: the copies
// of up to kStageRows rows (at most two ring chunks per array) are queued on
// the stream behind the sweeps that made them, the host waits once, then
// copies the rows into the caller's arrays.  (Direct copies into pageable
// caller memory cost one synchronous transfer per array and chunk.)
constexpr int64_t kStageRows = 256;

static int drain_records(isg_ising* H, int32_t* tslot, int64_t* bond, int64_t* mag,
                         int64_t row0) {
    const int RT = H->replicas_total;
    uint64_t n = H->records_made - H->records_done;
    if (n == 0) {
        ISG_CK(cudaStreamSynchronize(H->stream));
        return ISG_OK;
    }
    const size_t srows = (size_t)kStageRows * RT;
    if (!H->h_stage) ISG_CK(cudaMallocHost((void**)&H->h_stage, srows * 20));
    int64_t* st_b = reinterpret_cast<int64_t*>(H->h_stage);
    int64_t* st_m = st_b + srows;
    int32_t* st_t = reinterpret_cast<int32_t*>(st_m + srows);
    int64_t row = row0;
    while (n > 0) {
        const uint64_t batch = std::min<uint64_t>(n, (uint64_t)kStageRows);
        uint64_t done = H->records_done, left = batch;
        size_t srow = 0;
        while (left > 0) {
            const uint64_t slot = done % (uint64_t)H->ring_cap;
            const uint64_t chunk = std::min<uint64_t>(left, (uint64_t)H->ring_cap - slot);
            const size_t cnt = (size_t)chunk * RT, off = (size_t)slot * RT, so = srow * RT;
            ISG_CK(cudaMemcpyAsync(st_t + so, H->d_rec_t + off, cnt * sizeof(int32_t),
                                   cudaMemcpyDeviceToHost, H->stream));
            ISG_CK(cudaMemcpyAsync(st_b + so, H->d_rec_b + off, cnt * sizeof(int64_t),
                                   cudaMemcpyDeviceToHost, H->stream));
            ISG_CK(cudaMemcpyAsync(st_m + so, H->d_rec_m + off, cnt * sizeof(int64_t),
                                   cudaMemcpyDeviceToHost, H->stream));
            srow += chunk;
            done += chunk;
            left -= chunk;
        }
        ISG_CK(cudaStreamSynchronize(H->stream));
        const size_t cnt = (size_t)batch * RT;
        memcpy(tslot + (size_t)row * RT, st_t, cnt * sizeof(int32_t));
        memcpy(bond + (size_t)row * RT, st_b, cnt * sizeof(int64_t));
        memcpy(mag + (size_t)row * RT, st_m, cnt * sizeof(int64_t));
        H->records_done += batch;
        row += (int64_t)batch;
        n -= batch;
    }
    return ISG_OK;
}

}  // namespace isg

// ---------------------------------------------------------------- C ABI

extern "C" {

const char* isg_last_error(void) { return isg::g_last_error.c_str(); }
int isg_version(void) { return ISG_VERSION; }

int isg_ising_create(isg_ising** out, const int* sizes, int n_sizes, int replicas, int dim,
                     uint64_t seed) {
    if (!out) return fail(ISG_ERR_ARG, "isg_ising_create: out is NULL");
    *out = nullptr;
    if (!sizes || n_sizes < 1 || n_sizes > kMaxClasses)
        return fail(ISG_ERR_ARG, "isg_ising_create: need 1.." + std::to_string(kMaxClasses) +
                                     " sizes");
    if (replicas < 1 || replicas > kMaxReplicas)
        return fail(ISG_ERR_ARG, "isg_ising_create: replicas must be 1..1024");
    if (dim != 2 && dim != 3) return fail(ISG_ERR_ARG, "isg_ising_create: dim must be 2 or 3");
    for (int s = 0; s < n_sizes; ++s) {
        const int L = sizes[s];
        if (L < 2 || L > 1024)
            return fail(ISG_ERR_ARG, "isg_ising_create: size " + std::to_string(L) +
                                         " outside 2..1024");
        for (int q = 0; q < s; ++q)
            if (sizes[q] == L)
                return fail(ISG_ERR_ARG, "isg_ising_create: size " + std::to_string(L) +
                                             " listed twice (sizes share random streams)");
        if (L & 1)
            return fail(ISG_ERR_UNSUPPORTED,
                        "isg_ising_create: odd size " + std::to_string(L) +
                            " has no checkerboard colouring under periodic boundaries");
    }
    isg_ising* H = new (std::nothrow) isg_ising();
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_create: out of host memory");
    cudaGetDevice(&H->device);
    H->sms = num_sms(H->device);
    H->dim = dim;
    H->n_classes = n_sizes;
    H->R = replicas;
    H->replicas_total = n_sizes * replicas;
    H->seed = seed;
    H->sizes.assign(sizes, sizes + n_sizes);

    IsingParams& P = H->P;
    int64_t off = 0, task = 0, site = 0, sblk = 0;
    for (int s = 0; s < n_sizes; ++s) {
        IsingClass& C = P.cls[s];
        const int L = sizes[s];
        C.L = L;
        C.R = replicas;
        const int64_t nsite = dim == 3 ? (int64_t)L * L * L : (int64_t)L * L;
        C.plane_sites = (uint32_t)(nsite / 2);
        const bool pow2 = (L & (L - 1)) == 0;
        const int rw = L / 8;
        const bool words = pow2 && L >= 8 && L <= 256 && (32 % rw) == 0 &&
                           (C.plane_sites / 4) % 32 == 0;
        // other sizes with whole words per row and whole warp tasks per plane
        const bool gwords = !words && L % 8 == 0 && (C.plane_sites / 4) % 32 == 0;
        C.kind = words ? ((dim == 3 && L >= 32) ? kRolling : kFlat) : gwords ? kFlat : kSite;
        C.flat_gen = gwords ? 1 : 0;
        C.log2L = 0;
        while ((1 << C.log2L) < L) ++C.log2L;
        C.log2_rw = 0;
        if (words)
            while ((1 << C.log2_rw) < rw) ++C.log2_rw;
        C.tasks_per_plane = words || gwords ? C.plane_sites / 128 : 0;
        C.div_rw = make_div((uint32_t)std::max(1, rw));
        C.log2_tpp = 0;
        while (words && (1u << C.log2_tpp) < C.tasks_per_plane) ++C.log2_tpp;
        C.rep_base = s * replicas;
        C.spin_off = off;
        off += ((2 * (int64_t)C.plane_sites * replicas + 255) / 256) * 256;
        C.task_base = task;
        if (C.kind != kSite) task += (int64_t)C.tasks_per_plane * replicas;
        C.task_end = task;
        C.log2_groups = 0;
        C.log2_wpl = 1;
        // CTA tasks of the word kinds are laid out by layout_rolling / layout_flat
        C.ctask_base = C.ctask_end = 0;
        C.div_half = make_div((uint32_t)(L / 2));
        C.div_L = make_div((uint32_t)L);
        C.div_plane = make_div(C.plane_sites);
        C.plane_fast = (int64_t)C.plane_sites * replicas < ((int64_t)1 << 31) ? 1 : 0;
        C.site_base = site;
        if (C.kind == kSite) site += (int64_t)C.plane_sites * replicas;
        C.site_end = site;
        {
            const uint32_t S = dim == 3 ? (uint32_t)(L / 2) * (uint32_t)L : (uint32_t)(L / 2);
            C.s_nv = (uint32_t)((L + 3) / 4) * S;
            C.s_nb = (C.s_nv + 3) / 4;
            C.div_slab = make_div(S);
            C.div_nb = make_div(C.s_nb);
            C.sblk_fast = (int64_t)C.s_nb * replicas < ((int64_t)1 << 31) ? 1 : 0;
            C.sblk_base = sblk;
            if (C.kind == kSite) sblk += (int64_t)C.s_nb * replicas;
            C.sblk_end = sblk;
        }
    }
    // sentinel classes so the device class search always terminates
    for (int s = n_sizes; s < kMaxClasses; ++s) {
        P.cls[s] = P.cls[n_sizes - 1];
        P.cls[s].task_base = P.cls[s].task_end = INT64_MAX;
        P.cls[s].ctask_base = P.cls[s].ctask_end = INT64_MAX;
        P.cls[s].kind = -1;
        P.cls[s].site_base = P.cls[s].site_end = INT64_MAX;
        P.cls[s].sblk_base = P.cls[s].sblk_end = INT64_MAX;
    }
    P.n_classes = n_sizes;
    P.dim = dim;
    P.total_tasks = task;
    layout_rolling(H);
    layout_flat(H);
    P.total_sites = site;
    P.total_sblocks = sblk;
    P.seed = seed;
    for (int r = 0; r < 10; ++r) {
        P.rk0[r] = (uint32_t)seed + (uint32_t)r * kPhiloxW0;
        P.rk1[r] = (uint32_t)(seed >> 32) + (uint32_t)r * kPhiloxW1;
    }
    H->spin_bytes = off;

    const int RT = H->replicas_total;
    H->ring_cap = std::max<int64_t>(64, std::min<int64_t>(8192, (64ll << 20) / (20ll * RT)));
    auto cleanup = [&](int code) {
        isg_ising_destroy(H);
        return code;
    };
    cudaError_t e;
#define ALLOC(ptr, bytes)                                              \
    e = cudaMalloc((void**)&(ptr), (bytes));                           \
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMalloc"));
    ALLOC(H->d_spins, (size_t)off);
    ALLOC(H->d_thr, sizeof(uint32_t) * 16 * RT);
    ALLOC(H->d_thr8, sizeof(uint32_t) * 4 * RT);
    ALLOC(H->d_r2t, sizeof(int32_t) * RT);
    ALLOC(H->d_t2r, sizeof(int32_t) * RT);
    ALLOC(H->d_betas, sizeof(double) * RT);
    ALLOC(H->d_acc, sizeof(unsigned long long) * 2 * RT);
    ALLOC(H->d_ctrl, sizeof(unsigned long long) * (1 + 3 * kMaxClasses));
    ALLOC(H->d_rec_t, sizeof(int32_t) * (size_t)H->ring_cap * RT);
    ALLOC(H->d_rec_b, sizeof(long long) * (size_t)H->ring_cap * RT);
    ALLOC(H->d_rec_m, sizeof(long long) * (size_t)H->ring_cap * RT);
#undef ALLOC
    e = cudaStreamCreateWithFlags(&H->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaStreamCreateWithFlags"));
    H->stream = H->own_stream;

    P.spins = H->d_spins;
    P.thr = H->d_thr;
    P.thr8 = H->d_thr8;
    P.r2t = H->d_r2t;
    P.acc = H->d_acc;
    P.ctrl = H->d_ctrl;

    PostParams& Q = H->Q;
    Q.acc = H->d_acc;
    Q.r2t = H->d_r2t;
    Q.t2r = H->d_t2r;
    Q.betas = H->d_betas;
    Q.rec_t = H->d_rec_t;
    Q.rec_b = H->d_rec_b;
    Q.rec_m = H->d_rec_m;
    Q.ctrl = H->d_ctrl;
    Q.ring_cap = H->ring_cap;
    Q.seed = seed;
    Q.R = replicas;
    Q.n_classes = n_sizes;
    Q.replicas_total = RT;
    for (int s = 0; s < kMaxClasses; ++s) Q.L[s] = s < n_sizes ? sizes[s] : 0;

    std::vector<int32_t> ident(RT);
    for (int i = 0; i < RT; ++i) ident[i] = i % replicas;
#define CKC(call)                                                      \
    e = (call);                                                        \
    if (e != cudaSuccess) return cleanup(cuda_fail(e, #call));
    CKC(cudaMemsetAsync(H->d_spins, 0, (size_t)off, H->stream));
    CKC(cudaMemsetAsync(H->d_thr, 0, sizeof(uint32_t) * 16 * RT, H->stream));
    CKC(cudaMemsetAsync(H->d_thr8, 0, sizeof(uint32_t) * 4 * RT, H->stream));
    CKC(cudaMemsetAsync(H->d_acc, 0, sizeof(unsigned long long) * 2 * RT, H->stream));
    CKC(cudaMemsetAsync(H->d_ctrl, 0, sizeof(unsigned long long) * (1 + 3 * kMaxClasses),
                        H->stream));
    CKC(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                        H->stream));
    CKC(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                        H->stream));
    k_ising_init<<<H->sms * 4, 256, 0, H->stream>>>(H->P, dim);
    CKC(cudaGetLastError());
    CKC(cudaStreamSynchronize(H->stream));
#undef CKC
    int rc = configure_launch(H);
    if (rc != ISG_OK) return cleanup(rc);
    *out = H;
    return ISG_OK;
}

int isg_ising_destroy(isg_ising* H) {
    if (!H) return ISG_OK;
    cudaSetDevice(H->device);
    // A caller's stream may already be gone: wait for the device instead.
    if (H->stream == H->own_stream) {
        if (H->stream) cudaStreamSynchronize(H->stream);
    } else {
        cudaDeviceSynchronize();
    }
    destroy_graph(H);
    cudaFree(H->d_spins);
    cudaFree(H->d_thr);
    cudaFree(H->d_thr8);
    cudaFree(H->d_r2t);
    cudaFree(H->d_t2r);
    cudaFree(H->d_betas);
    cudaFree(H->d_acc);
    cudaFree(H->d_ctrl);
    cudaFree(H->d_rec_t);
    cudaFree(H->d_rec_b);
    if (H->h_stage) cudaFreeHost(H->h_stage);
    cudaFree(H->d_rec_m);
    cudaFree(H->d_sched_tab);
    cudaFree(H->d_sched);
    cudaFree(H->d_srec);
    cudaFree(H->d_srec_t);
    cudaFree(H->d_pt_scratch);
    cudaFree(H->d_hist);
    cudaFree(H->d_hist_rng);
    if (H->own_stream) cudaStreamDestroy(H->own_stream);
    delete H;
    return ISG_OK;
}

int isg_ising_set_stream(isg_ising* H, void* stream) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_stream: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->stream = stream ? (cudaStream_t)stream : H->own_stream;
    return ISG_OK;
}

}  // extern "C"

namespace isg {
// The 16-entry acceptance table of temperature T: entry own_down*8 + n_down.
static void threshold_table(int dim, double T, double J, double hfield, uint32_t* thr) {
    const double beta = 1.0 / T;
    for (int e = 0; e < 16; ++e) thr[e] = 0u;
    for (int od = 0; od < 2; ++od) {
        const double sgn = od ? -1.0 : 1.0;
        for (int nd = 0; nd <= 2 * dim; ++nd) {
            const double nb = (double)(2 * dim - 2 * nd);
            const double dE = 2.0 * sgn * (J * nb + hfield);
            uint32_t t;
            if (dE <= 0.0) {
                t = 0xFFFFFFFFu;
            } else {
                double f = std::floor(std::exp(-beta * dE) * 4294967296.0);
                if (f < 1.0) f = 1.0;
                t = (uint32_t)(f - 1.0);
            }
            thr[od * 8 + nd] = t;
        }
    }
}

// Uploads the per-slot thresholds ([slots][16]) and their coarse bytes for the
// word kernels ([slots][4]: byte own_down*8 + n_down = 0x80 for 0xFFFFFFFF,
// else threshold >> 25).
static int upload_thresholds(isg_ising* H, const std::vector<uint32_t>& thr) {
    const size_t n = thr.size() / 16;
    std::vector<uint32_t> t8(4 * n, 0u);
    for (size_t i = 0; i < n; ++i)
        for (int e = 0; e < 16; ++e) {
            const uint32_t t = thr[i * 16 + (size_t)e];
            const uint32_t b = t == 0xFFFFFFFFu ? 0x80u : t >> 25;
            t8[4 * i + (size_t)(e >> 2)] |= b << (8 * (e & 3));
        }
    ISG_CK(cudaMemcpyAsync(H->d_thr, thr.data(), thr.size() * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_thr8, t8.data(), t8.size() * sizeof(uint32_t),
                           cudaMemcpyHostToDevice, H->stream));
    return ISG_OK;
}
}  // namespace isg

namespace isg {
static int pt_resident(isg_ising* H, int64_t n_sweeps, int ee, int me, int32_t* tslot,
                       int64_t* bond, int64_t* mag, int64_t max_records, int64_t* n_records);
}  // namespace isg

extern "C" {

int isg_ising_set_temperatures(isg_ising* H, const double* temps, double J, double hfield) {
    if (!H || !temps) return fail(ISG_ERR_ARG, "isg_ising_set_temperatures: NULL argument");
    cudaSetDevice(H->device);
    const int RT = H->replicas_total;
    std::vector<uint32_t> thr(16 * (size_t)RT, 0u);
    std::vector<double> betas(RT);
    for (int i = 0; i < RT; ++i) {
        if (!(temps[i] > 0.0) || !std::isfinite(temps[i]))
            return fail(ISG_ERR_ARG, "isg_ising_set_temperatures: temperatures must be positive");
        betas[i] = 1.0 / temps[i];
        threshold_table(H->dim, temps[i], J, hfield, &thr[(size_t)i * 16]);
    }
    std::vector<int32_t> ident(RT);
    for (int i = 0; i < RT; ++i) ident[i] = i % H->R;
    {
        const int rc = upload_thresholds(H, thr);
        if (rc) return rc;
    }
    ISG_CK(cudaMemcpyAsync(H->d_betas, betas.data(), betas.size() * sizeof(double),
                           cudaMemcpyHostToDevice, H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_r2t, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_t2r, ident.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    // graph nodes hold J and h by value; thresholds and maps are read from
    // device memory, so the graphs survive a change of temperatures alone
    if (!H->temps_set || J != H->J || hfield != H->h) destroy_graph(H);
    H->J = J;
    H->h = hfield;
    H->Q.J = J;
    H->Q.h = hfield;
    H->temps_set = true;
    return ISG_OK;
}

int isg_ising_step(isg_ising* H, int64_t n_sweeps) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_step: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_ising_step: temperatures not set");
    if (n_sweeps < 0) return fail(ISG_ERR_ARG, "isg_ising_step: negative sweep count");
    if (n_sweeps == 0) return ISG_OK;
    cudaSetDevice(H->device);
    int64_t done = 0;
    if (n_sweeps >= kStepGraphSweeps && !H->step_graph) {
        cudaGraph_t g = nullptr;
        ISG_CK(cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal));
        for (int j = 0; j < kStepGraphSweeps; ++j) {
            launch_half(H, 0, j, 0);
            launch_half(H, 1, j, 0);
        }
        launch_post(H, 0, 0, 0, 0, kStepGraphSweeps);
        cudaError_t e = cudaStreamEndCapture(H->stream, &g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&H->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            H->step_graph = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate");
        }
    }
    for (; n_sweeps - done >= kStepGraphSweeps; done += kStepGraphSweeps)
        ISG_CK(cudaGraphLaunch(H->step_graph, H->stream));
    while (done < n_sweeps) {
        const int chunk = (int)std::min<int64_t>(n_sweeps - done, 1 << 20);
        for (int j = 0; j < chunk; ++j) {
            launch_half(H, 0, j, 0);
            launch_half(H, 1, j, 0);
        }
        launch_post(H, 0, 0, 0, 0, chunk);
        done += chunk;
    }
    H->gsweep += (uint64_t)n_sweeps;
    return check_launch("isg_ising_step");
}

int isg_ising_measure(isg_ising* H, int64_t* bond, int64_t* mag) {
    if (!H || !bond || !mag) return fail(ISG_ERR_ARG, "isg_ising_measure: NULL argument");
    cudaSetDevice(H->device);
    const int RT = H->replicas_total;
    ISG_CK(cudaMemsetAsync(H->d_acc, 0, sizeof(unsigned long long) * 2 * RT, H->stream));
    launch_half(H, 1, 0, 2);
    int rc = check_launch("isg_ising_measure");
    if (rc) return rc;
    std::vector<unsigned long long> acc(2 * (size_t)RT);
    ISG_CK(cudaMemcpyAsync(acc.data(), H->d_acc, acc.size() * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    for (int i = 0; i < RT; ++i) {
        bond[i] = (int64_t)acc[2 * i];
        mag[i] = (int64_t)acc[2 * i + 1];
    }
    return ISG_OK;
}

int isg_ising_exchange(isg_ising* H, int parity, int64_t* accepted) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_exchange: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_ising_exchange: temperatures not set");
    cudaSetDevice(H->device);
    const int NC = H->n_classes;
    std::vector<unsigned long long> before(NC), after(NC);
    ISG_CK(cudaMemcpyAsync(before.data(), H->d_ctrl + 1 + 2 * NC, NC * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, H->stream));
    launch_post(H, 0, 1, parity, 1, 0);
    int rc = check_launch("isg_ising_exchange");
    if (rc) return rc;
    ISG_CK(cudaMemcpyAsync(after.data(), H->d_ctrl + 1 + 2 * NC, NC * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    if (accepted)
        for (int s = 0; s < NC; ++s) accepted[s] = (int64_t)(after[s] - before[s]);
    return ISG_OK;
}

int isg_ising_get_r2t(isg_ising* H, int32_t* r2t) {
    if (!H || !r2t) return fail(ISG_ERR_ARG, "isg_ising_get_r2t: NULL argument");
    cudaSetDevice(H->device);
    ISG_CK(cudaMemcpyAsync(r2t, H->d_r2t, sizeof(int32_t) * H->replicas_total,
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

int isg_ising_set_r2t(isg_ising* H, const int32_t* r2t) {
    if (!H || !r2t) return fail(ISG_ERR_ARG, "isg_ising_set_r2t: NULL argument");
    cudaSetDevice(H->device);
    const int R = H->R, RT = H->replicas_total;
    std::vector<int32_t> t2r(RT, -1);
    for (int s = 0; s < H->n_classes; ++s)
        for (int r = 0; r < R; ++r) {
            const int t = r2t[s * R + r];
            if (t < 0 || t >= R || t2r[s * R + t] != -1)
                return fail(ISG_ERR_ARG, "isg_ising_set_r2t: not a permutation per size");
            t2r[s * R + t] = r;
        }
    ISG_CK(cudaMemcpyAsync(H->d_r2t, r2t, sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaMemcpyAsync(H->d_t2r, t2r.data(), sizeof(int32_t) * RT, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

static int spin_geometry(isg_ising* H, int s, int r, int64_t* nsite, int64_t* base) {
    if (s < 0 || s >= H->n_classes || r < 0 || r >= H->R)
        return fail(ISG_ERR_ARG, "spin access: size index or replica out of range");
    const IsingClass& C = H->P.cls[s];
    *nsite = 2 * (int64_t)C.plane_sites;
    *base = C.spin_off + (int64_t)r * *nsite;
    return ISG_OK;
}

int isg_ising_get_spins(isg_ising* H, int s, int r, int8_t* out) {
    if (!H || !out) return fail(ISG_ERR_ARG, "isg_ising_get_spins: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    int rc = spin_geometry(H, s, r, &n, &base);
    if (rc) return rc;
    std::vector<uint8_t> planes((size_t)n);
    ISG_CK(cudaMemcpyAsync(planes.data(), H->d_spins + base, (size_t)n, cudaMemcpyDeviceToHost,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    const int L = H->sizes[s];
    const int64_t half = n / 2;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t x = i % L, y = (i / L) % L, z = H->dim == 3 ? i / ((int64_t)L * L) : 0;
        const int c = (int)((x + y + z) & 1);
        out[i] = planes[(size_t)(c * half + (i >> 1))] ? (int8_t)-1 : (int8_t)1;
    }
    return ISG_OK;
}

int isg_ising_set_spins(isg_ising* H, int s, int r, const int8_t* in) {
    if (!H || !in) return fail(ISG_ERR_ARG, "isg_ising_set_spins: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    int rc = spin_geometry(H, s, r, &n, &base);
    if (rc) return rc;
    std::vector<uint8_t> planes((size_t)n);
    const int L = H->sizes[s];
    const int64_t half = n / 2;
    for (int64_t i = 0; i < n; ++i) {
        if (in[i] != 1 && in[i] != -1)
            return fail(ISG_ERR_ARG, "isg_ising_set_spins: spins must be +1 or -1");
        const int64_t x = i % L, y = (i / L) % L, z = H->dim == 3 ? i / ((int64_t)L * L) : 0;
        const int c = (int)((x + y + z) & 1);
        planes[(size_t)(c * half + (i >> 1))] = in[i] < 0 ? 1 : 0;
    }
    ISG_CK(cudaMemcpyAsync(H->d_spins + base, planes.data(), (size_t)n, cudaMemcpyHostToDevice,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

int isg_ising_load_natural(isg_ising* H, int s, int r, const int8_t* d_nat) {
    if (!H || !d_nat) return fail(ISG_ERR_ARG, "isg_ising_load_natural: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    int rc = spin_geometry(H, s, r, &n, &base);
    if (rc) return rc;
    k_ising_nat_to_planes<<<(int)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, H->stream>>>(
        H->d_spins + base, d_nat, H->sizes[s], H->dim, (uint32_t)(n / 2));
    return check_launch("isg_ising_load_natural");
}

int isg_ising_store_natural(isg_ising* H, int s, int r, int8_t* d_nat) {
    if (!H || !d_nat) return fail(ISG_ERR_ARG, "isg_ising_store_natural: NULL argument");
    cudaSetDevice(H->device);
    int64_t n, base;
    int rc = spin_geometry(H, s, r, &n, &base);
    if (rc) return rc;
    k_ising_planes_to_nat<<<(int)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, H->stream>>>(
        H->d_spins + base, d_nat, H->sizes[s], H->dim, (uint32_t)(n / 2));
    return check_launch("isg_ising_store_natural");
}

int isg_ising_store_natural_all(isg_ising* H, int s, int8_t* d_nat) {
    if (!H || !d_nat) return fail(ISG_ERR_ARG, "isg_ising_store_natural_all: NULL argument");
    if (s < 0 || s >= H->n_classes)
        return fail(ISG_ERR_ARG, "isg_ising_store_natural_all: bad size index");
    cudaSetDevice(H->device);
    for (int r = 0; r < H->R; ++r) {
        int64_t n, base;
        int rc = spin_geometry(H, s, r, &n, &base);
        if (rc) return rc;
        k_ising_planes_to_nat<<<(int)std::min<int64_t>(1024, (n + 255) / 256), 256, 0,
                                H->stream>>>(H->d_spins + base, d_nat + (size_t)r * n,
                                             H->sizes[s], H->dim, (uint32_t)(n / 2));
    }
    return check_launch("isg_ising_store_natural_all");
}

int isg_ising_reset_sampling(isg_ising* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_reset_sampling: NULL handle");
    cudaSetDevice(H->device);
    const int NC = H->n_classes;
    ISG_CK(cudaMemsetAsync(H->d_ctrl + 1, 0, sizeof(unsigned long long) * 3 * NC, H->stream));
    ISG_CK(cudaMemsetAsync(H->d_acc, 0, sizeof(unsigned long long) * 2 * H->replicas_total,
                           H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->ksample = 0;
    H->records_done = H->records_made = 0;
    return ISG_OK;
}

int isg_ising_pt_run(isg_ising* H, int64_t n_sweeps, int ee, int me, int32_t* tslot,
                     int64_t* bond, int64_t* mag, int64_t max_records, int64_t* n_records) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_pt_run: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_ising_pt_run: temperatures not set");
    if (n_sweeps < 0 || ee < 1 || me < 1)
        return fail(ISG_ERR_ARG, "isg_ising_pt_run: need n_sweeps >= 0, exchange_every >= 1, "
                                 "measure_every >= 1");
    cudaSetDevice(H->device);
    // keep: records stay in the device ring (newest ring_cap rows), no host sync
    const bool keep = tslot == nullptr && bond == nullptr && mag == nullptr;
    const uint64_t k0 = H->ksample;
    const uint64_t need = (k0 + (uint64_t)n_sweeps) / (uint64_t)me - k0 / (uint64_t)me;
    if (!keep && need > 0 && (!tslot || !bond || !mag || max_records < (int64_t)need))
        return fail(ISG_ERR_ARG, "isg_ising_pt_run: record arrays hold " +
                                     std::to_string(max_records) + " rows, " +
                                     std::to_string(need) + " needed");
    if (n_records) *n_records = 0;
    if (!keep && n_sweeps > 0) {
        // small lattices: the whole run in the resident kernel (1: not eligible)
        const int rc = pt_resident(H, n_sweeps, ee, me, tslot, bond, mag, max_records, n_records);
        if (rc != 1) return rc;
    }
    const int64_t g = gcd64(ee, me);
    const int64_t lcm = (int64_t)ee / g * me;
    const int period = lcm <= 1000 ? (int)lcm : 0;
    const int rec_per_period = period ? period / me : 0;
    const bool use_graph = period > 0 && rec_per_period <= H->ring_cap / 2;
    int64_t done = 0, row = 0;
    while (done < n_sweeps) {
        const uint64_t k = H->ksample;
        const int64_t left = n_sweeps - done;
        const uint64_t pending = H->records_made - H->records_done;
        const bool whole = use_graph && (k % (uint64_t)period) == 0 && left >= period;
        const uint64_t adds = whole ? (uint64_t)rec_per_period : 1u;
        if (pending + adds > (uint64_t)H->ring_cap) {
            if (keep) {
                H->records_done = H->records_made + adds - (uint64_t)H->ring_cap;
            } else {
                int rc = drain_records(H, tslot, bond, mag, row);
                if (rc) return rc;
                row += (int64_t)pending;
                continue;
            }
        }
        if (whole) {
            if (!H->graph || H->graph_ee != ee || H->graph_me != me || H->graph_period != period) {
                int rc = build_graph(H, ee, me, period);
                if (rc) return rc;
            }
            ISG_CK(cudaGraphLaunch(H->graph, H->stream));
            H->ksample += (uint64_t)period;
            H->gsweep += (uint64_t)period;
            H->records_made += (uint64_t)rec_per_period;
            done += period;
        } else {
            const bool do_m = ((k + 1) % (uint64_t)me) == 0;
            issue_sample_sweep(H, k, 0, ee, me, 1);
            int rc = check_launch("isg_ising_pt_run");
            if (rc) return rc;
            H->ksample += 1;
            H->gsweep += 1;
            if (do_m) H->records_made += 1;
            done += 1;
        }
    }
    if (keep) return check_launch("isg_ising_pt_run");
    const uint64_t pending = H->records_made - H->records_done;
    int rc = drain_records(H, tslot, bond, mag, row);
    if (rc) return rc;
    row += (int64_t)pending;
    if (n_records) *n_records = row;
    return ISG_OK;
}

int isg_ising_read_records(isg_ising* H, int32_t* tslot, int64_t* bond, int64_t* mag,
                           int64_t max_records, int64_t* n_records) {
    if (!H || !tslot || !bond || !mag || !n_records)
        return fail(ISG_ERR_ARG, "isg_ising_read_records: NULL argument");
    cudaSetDevice(H->device);
    const uint64_t pending = H->records_made - H->records_done;
    if ((int64_t)pending > max_records)
        H->records_done = H->records_made - (uint64_t)std::max<int64_t>(max_records, 0);
    const uint64_t n = H->records_made - H->records_done;
    int rc = drain_records(H, tslot, bond, mag, 0);
    if (rc) return rc;
    *n_records = (int64_t)n;
    return ISG_OK;
}

int isg_ising_get_accepted(isg_ising* H, int64_t* accepted) {
    if (!H || !accepted) return fail(ISG_ERR_ARG, "isg_ising_get_accepted: NULL argument");
    cudaSetDevice(H->device);
    const int NC = H->n_classes;
    std::vector<unsigned long long> a(NC);
    ISG_CK(cudaMemcpyAsync(a.data(), H->d_ctrl + 1 + 2 * NC, NC * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    for (int s = 0; s < NC; ++s) accepted[s] = (int64_t)a[s];
    return ISG_OK;
}

int isg_ising_get_sweep(isg_ising* H, uint64_t* sweep) {
    if (!H || !sweep) return fail(ISG_ERR_ARG, "isg_ising_get_sweep: NULL argument");
    cudaSetDevice(H->device);
    unsigned long long v = 0;
    ISG_CK(cudaMemcpyAsync(&v, H->d_ctrl, sizeof(v), cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    *sweep = v;
    return ISG_OK;
}

int isg_ising_sync(isg_ising* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_sync: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    return check_launch("isg_ising_sync");
}

int isg_ising_set_launch(isg_ising* H, int threads, int blocks_per_sm) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_launch: NULL handle");
    if (threads != 64 && threads != 128 && threads != 256 && threads != 512)
        return fail(ISG_ERR_ARG, "isg_ising_set_launch: threads must be 64, 128, 256 or 512");
    if (blocks_per_sm < 0 || blocks_per_sm > 64)
        return fail(ISG_ERR_ARG, "isg_ising_set_launch: blocks_per_sm must be 0..64");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->threads = threads;
    H->blocks_per_sm = blocks_per_sm;
    destroy_graph(H);
    return configure_launch(H);
}

// Runs n sweeps' worth of half-sweeps on the live buffers, timing each launch,
// then restores the spins and the sweep counter.
static int timed_halfsweeps(isg_ising* H, int n_launches, float* avg_ms) {
    uint8_t* backup = nullptr;
    ISG_CK(cudaMalloc((void**)&backup, (size_t)H->spin_bytes));
    unsigned long long ctrl0 = 0;
    cudaError_t e = cudaMemcpyAsync(backup, H->d_spins, (size_t)H->spin_bytes,
                                    cudaMemcpyDeviceToDevice, H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&ctrl0, H->d_ctrl, sizeof(ctrl0), cudaMemcpyDeviceToHost, H->stream);
    cudaEvent_t a = nullptr, b = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float total = 0.f;
    for (int i = 0; i < n_launches && e == cudaSuccess; ++i) {
        e = cudaEventRecord(a, H->stream);
        launch_half(H, i & 1, i >> 1, 0);
        if (e == cudaSuccess) e = cudaEventRecord(b, H->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        total += ms;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_spins, backup, (size_t)H->spin_bytes, cudaMemcpyDeviceToDevice,
                            H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_ctrl, &ctrl0, sizeof(ctrl0), cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(backup);
    if (e != cudaSuccess) return cuda_fail(e, "timed_halfsweeps");
    *avg_ms = n_launches > 0 ? total / (float)n_launches : 0.f;
    return ISG_OK;
}

int isg_ising_time_halfsweep(isg_ising* H, int n_launches, float* avg_ms) {
    if (!H || !avg_ms || n_launches < 1)
        return fail(ISG_ERR_ARG, "isg_ising_time_halfsweep: bad argument");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_ising_time_halfsweep: temperatures not set");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    return timed_halfsweeps(H, n_launches, avg_ms);
}

// The half-sweeps as they run inside a PT cycle: n_launches launches (colours
// alternating, as n_launches/2 sweeps) captured as one CUDA graph, each replay
// preceded by a write of flush_bytes (so the first launch of a replay starts
// from a cold L2, like the first launch of a timed PT step), timed with events
// on the handle's stream around the graph alone.  Spins and sweep counter are
// restored afterwards.
int isg_ising_time_halfsweep_graph(isg_ising* H, int n_launches, int64_t flush_bytes,
                                   int replays, float* avg_ms) {
    if (!H || !avg_ms || n_launches < 1 || n_launches > 4096 || flush_bytes < 0 || replays < 1)
        return fail(ISG_ERR_ARG, "isg_ising_time_halfsweep_graph: bad argument");
    if (!H->temps_set)
        return fail(ISG_ERR_STATE, "isg_ising_time_halfsweep_graph: temperatures not set");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    uint8_t* backup = nullptr;
    uint8_t* flush = nullptr;
    ISG_CK(cudaMalloc((void**)&backup, (size_t)H->spin_bytes));
    cudaError_t e = cudaSuccess;
    if (flush_bytes > 0) e = cudaMalloc((void**)&flush, (size_t)flush_bytes);
    unsigned long long ctrl0 = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(backup, H->d_spins, (size_t)H->spin_bytes, cudaMemcpyDeviceToDevice,
                            H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&ctrl0, H->d_ctrl, sizeof(ctrl0), cudaMemcpyDeviceToHost, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(H->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int i = 0; i < n_launches; ++i) launch_half(H, i & 1, i >> 1, 0);
        e = cudaStreamEndCapture(H->stream, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    cudaEvent_t a = nullptr, b = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    float total = 0.f;
    for (int rep = 0; rep <= replays && e == cudaSuccess; ++rep) {  // replay 0 warms up
        if (flush) e = cudaMemsetAsync(flush, rep & 0xFF, (size_t)flush_bytes, H->stream);
        if (e == cudaSuccess) e = cudaEventRecord(a, H->stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(ge, H->stream);
        if (e == cudaSuccess) e = cudaEventRecord(b, H->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        if (rep > 0) total += ms;
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_spins, backup, (size_t)H->spin_bytes, cudaMemcpyDeviceToDevice,
                            H->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(H->d_ctrl, &ctrl0, sizeof(ctrl0), cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    cudaFree(backup);
    if (flush) cudaFree(flush);
    if (e != cudaSuccess) return cuda_fail(e, "isg_ising_time_halfsweep_graph");
    *avg_ms = total / (float)((int64_t)replays * n_launches);
    return ISG_OK;
}

int isg_ising_set_cache_prefetch(isg_ising* H, int level, int planes) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_cache_prefetch: NULL handle");
    if (planes < 0 || planes > 16 || (level != 1 && level != 2))
        return fail(ISG_ERR_ARG, "isg_ising_set_cache_prefetch: level must be 1 or 2, planes 0..16");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->P.l2_ahead = planes;
    H->P.pf_level = level;
    H->cache_pf_set = true;
    destroy_graph(H);
    return ISG_OK;
}

int isg_ising_set_resident_pt(isg_ising* H, int enable) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_resident_pt: NULL handle");
    H->resident_pt = enable != 0;
    return ISG_OK;
}

int isg_ising_set_dependent_launch(isg_ising* H, int enable) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_dependent_launch: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->pdl = enable != 0;
    destroy_graph(H);
    return ISG_OK;
}

int isg_ising_set_words_per_lane(isg_ising* H, int words) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_words_per_lane: NULL handle");
    if (words != 2 && words != 4)
        return fail(ISG_ERR_ARG, "isg_ising_set_words_per_lane: words must be 2 or 4");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->wpl_max = words;
    layout_rolling(H);
    layout_flat(H);
    destroy_graph(H);
    return configure_launch(H);
}

int isg_ising_set_prefetch(isg_ising* H, int depth) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_set_prefetch: NULL handle");
    if (depth < 0 || depth > 3) return fail(ISG_ERR_ARG, "isg_ising_set_prefetch: depth must be 0..3");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    H->prefetch = depth;
    destroy_graph(H);
    return configure_launch(H);
}

int isg_ising_autotune(isg_ising* H, int* best) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_autotune: NULL handle");
    if (!H->temps_set) return fail(ISG_ERR_STATE, "isg_ising_autotune: temperatures not set");
    cudaSetDevice(H->device);
    const int thr_opts[] = {128, 256, 512};
    const int bps_opts[] = {1, 2, 4, 8, 16, 0};
    float best_ms = 1e30f;
    int bt = H->threads, bb = H->blocks_per_sm, bp = H->prefetch;
    // prefetch forms: registers one or two planes ahead; with four words per
    // lane also the shared-memory ring
    const int npf = H->dim == 3 ? (H->wmax == 4 ? 3 : 2) : 1;
    for (int pf = 1; pf <= npf; ++pf)
        for (int t : thr_opts)
            for (int b : bps_opts) {
                if (b > 0 && b * t > 2048) continue;
                H->prefetch = pf;
                int rc = isg_ising_set_launch(H, t, b);
                if (rc) return rc;
                float ms = 0.f;
                rc = timed_halfsweeps(H, 2, &ms);  // warm
                if (rc) return rc;
                rc = timed_halfsweeps(H, 8, &ms);
                if (rc) return rc;
                if (ms < best_ms) {
                    best_ms = ms;
                    bt = t;
                    bb = b;
                    bp = pf;
                }
            }
    H->prefetch = bp;
    int rc = isg_ising_set_launch(H, bt, bb);
    if (rc) return rc;
    if (best) {
        best[0] = bt;
        best[1] = bb;
        best[2] = bp;
    }
    return ISG_OK;
}

int isg_ising_sites_per_halfsweep(isg_ising* H, int64_t* sites) {
    if (!H || !sites) return fail(ISG_ERR_ARG, "isg_ising_sites_per_halfsweep: NULL argument");
    int64_t n = 0;
    for (int s = 0; s < H->n_classes; ++s) n += (int64_t)H->P.cls[s].plane_sites * H->R;
    *sites = n;
    return ISG_OK;
}

// ------------------------------------------------------------ schedules

}  // extern "C"

namespace isg {

// Lattices up to this many sites per colour plane run whole schedules in the
// cluster-resident kernel; larger ones sweep with the half-sweep kernels.
constexpr uint32_t kResidentMaxPlane = 1u << 16;

static int grow(void** p, int64_t* cap, int64_t need_bytes) {
    if (*cap >= need_bytes) return ISG_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, (size_t)need_bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    *cap = need_bytes;
    return ISG_OK;
}

// Every slot's table (and exchange beta) set to temperature T.
static int all_slots_to(isg_ising* H, double T) {
    const int RT = H->replicas_total;
    std::vector<uint32_t> thr(16 * (size_t)RT);
    threshold_table(H->dim, T, H->J, H->h, thr.data());
    for (int i = 1; i < RT; ++i) std::copy(thr.begin(), thr.begin() + 16, thr.begin() + 16 * i);
    std::vector<double> betas(RT, 1.0 / T);
    {
        const int rc = upload_thresholds(H, thr);
        if (rc) return rc;
    }
    ISG_CK(cudaMemcpyAsync(H->d_betas, betas.data(), betas.size() * sizeof(double),
                           cudaMemcpyHostToDevice, H->stream));
    return ISG_OK;
}

static int64_t count_rows(int64_t n, int every, int phase) {
    if (every <= 0 || n <= phase) return 0;
    return (n - 1 - phase) / every + 1;
}

static int copy_records(isg_ising* H, const unsigned long long* d_rec, int64_t rows,
                        int64_t row0, int64_t* bond, int64_t* mag) {
    const int RT = H->replicas_total;
    std::vector<unsigned long long> buf((size_t)rows * RT * 2);
    ISG_CK(cudaMemcpyAsync(buf.data(), d_rec, buf.size() * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    for (int64_t row = 0; row < rows; ++row)
        for (int l = 0; l < RT; ++l) {
            const size_t o = ((size_t)row * RT + l) * 2;
            bond[(size_t)(row0 + row) * RT + l] = (int64_t)buf[o];
            mag[(size_t)(row0 + row) * RT + l] = (int64_t)buf[o + 1];
        }
    return ISG_OK;
}

// Launch shape of the resident kernel: the largest cluster that fits a GPC
// (16, 8, 4, 2 or 1 CTAs of kResidentThreads), each CTA holding a power-of-two
// chunk (>= 256 sites where the cluster has several CTAs) of both colour
// planes.  Sets cfg (grid, block, shared memory, cluster attribute in attr[0]),
// Q.cs and Q.log2_chunk; *active = clusters that can be resident at once.
static bool resident_config(isg_ising* H, cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr,
                            ResidentParams& Q, const void* kfun, uint32_t max_plane, int* active) {
    const int RT = H->replicas_total;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    cfg.blockDim = dim3(kResidentThreads, 1, 1);
    cfg.stream = H->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    *active = 0;
    for (int target = 16; target >= 1; target /= 2) {
        int lc = 0;
        while ((1u << lc) * (uint32_t)target < max_plane) ++lc;
        if (lc < 8 && target > 1) continue;  // fewer than 256 sites per CTA: smaller cluster
        const int cs = (int)((max_plane + (1u << lc) - 1) >> lc);
        const size_t smem = (size_t)2 << lc;
        if (smem > 200 * 1024) break;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(kfun, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        Q.cs = cs;
        Q.log2_chunk = lc;
        cfg.gridDim = dim3((unsigned)(RT * cs), 1, 1);
        cfg.dynamicSmemBytes = smem;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        int a = 0;
        if (cudaOccupancyMaxActiveClusters(&a, kfun, &cfg) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (a > 0) {
            *active = a;
            return true;
        }
    }
    return false;
}

static int schedule_resident(isg_ising* H, const double* temps, int64_t n_sweeps, int every,
                             int phase, int64_t* bond, int64_t* mag) {
    const int RT = H->replicas_total;
    uint32_t max_plane = 0;
    for (int s = 0; s < H->n_classes; ++s) max_plane = std::max(max_plane, H->P.cls[s].plane_sites);
    // about 256 sites per CTA and colour plane (power-of-two chunks), at most
    // 16 CTAs per cluster (non-portable sizes above 8 where the GPU allows them)
    const void* kfun = H->dim == 3 ? (const void*)k_ising_resident<3>
                                   : (const void*)k_ising_resident<2>;
    if (cudaFuncSetAttribute(kfun, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
        cudaSuccess)
        cudaGetLastError();  // portable sizes only; the occupancy check below shrinks them
    // distinct temperatures -> tables
    std::vector<uint32_t> tabs;
    std::vector<int32_t> idx;
    if (temps) {
        std::vector<std::pair<double, int32_t>> seen;
        idx.resize((size_t)n_sweeps);
        for (int64_t k = 0; k < n_sweeps; ++k) {
            if (k > 0 && temps[k] == temps[k - 1]) {
                idx[k] = idx[k - 1];
                continue;
            }
            int32_t found = -1;
            if (!seen.empty() && seen.back().first == temps[k]) found = seen.back().second;
            if (found < 0) {
                found = (int32_t)(tabs.size() / 16);
                tabs.resize(tabs.size() + 16);
                threshold_table(H->dim, temps[k], H->J, H->h, &tabs[tabs.size() - 16]);
                seen.emplace_back(temps[k], found);
            }
            idx[k] = found;
        }
        int rc = grow((void**)&H->d_sched_tab, &H->sched_tab_cap,
                      (int64_t)tabs.size() * (int64_t)sizeof(uint32_t));
        if (rc) return rc;
        rc = grow((void**)&H->d_sched, &H->sched_cap, n_sweeps * (int64_t)sizeof(int32_t));
        if (rc) return rc;
        ISG_CK(cudaMemcpyAsync(H->d_sched_tab, tabs.data(), tabs.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, H->stream));
        ISG_CK(cudaMemcpyAsync(H->d_sched, idx.data(), idx.size() * sizeof(int32_t),
                               cudaMemcpyHostToDevice, H->stream));
    }
    // launches of whole multiples of `every` sweeps keep the record phase
    const int64_t span = every > 0 ? std::max<int64_t>(every, ((int64_t)1 << 16) / every * every)
                                   : ((int64_t)1 << 16);
    const int64_t max_rows = count_rows(std::min(span, n_sweeps), every, phase);
    if (max_rows > 0) {
        int rc = grow((void**)&H->d_srec, &H->srec_cap,
                      max_rows * RT * 2 * (int64_t)sizeof(unsigned long long));
        if (rc) return rc;
    }
    int64_t row0 = 0;
    for (int64_t k0 = 0; k0 < n_sweeps; k0 += span) {
        const int64_t n = std::min(span, n_sweeps - k0);
        const int64_t rows = count_rows(n, every, phase);
        if (rows > 0)
            ISG_CK(cudaMemsetAsync(H->d_srec, 0, rows * RT * 2 * sizeof(unsigned long long),
                                   H->stream));
        ResidentParams Q{};
        Q.tables = temps ? H->d_sched_tab : H->d_thr;
        Q.sched = temps ? H->d_sched + k0 : nullptr;
        Q.rec = H->d_srec;
        Q.sweep0 = H->gsweep;
        Q.n_sweeps = n;
        Q.measure_every = rows > 0 ? every : 0;
        Q.measure_phase = phase;
        Q.lattices = RT;
        for (int c = 0; c < kMaxClasses; ++c) {
            const int L = H->P.cls[c < H->n_classes ? c : 0].L;
            Q.div_half[c] = make_div((uint32_t)(L / 2));
            Q.div_L[c] = make_div((uint32_t)L);
        }
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[2];
        int active = 0;
        if (!resident_config(H, cfg, attr, Q, kfun, max_plane, &active) || active < 1)
            return fail(ISG_ERR_UNSUPPORTED, "isg_ising_run_schedule: no cluster shape fits");
        cudaError_t e = H->dim == 3 ? cudaLaunchKernelEx(&cfg, k_ising_resident<3>, H->P, Q)
                                    : cudaLaunchKernelEx(&cfg, k_ising_resident<2>, H->P, Q);
        if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchKernelEx(k_ising_resident)");
        launch_post(H, 0, 0, 0, 0, (int)n);  // device sweep counter
        H->gsweep += (uint64_t)n;
        int rc = check_launch("isg_ising_run_schedule");
        if (rc) return rc;
        if (rows > 0) {
            rc = copy_records(H, H->d_srec, rows, row0, bond, mag);
            if (rc) return rc;
            row0 += rows;
        }
    }
    return ISG_OK;
}

// Larger lattices: half-sweep kernels sweep by sweep, the measurement fused
// into the second half-sweep of a recorded sweep.
// PT sampling of small lattices (at most 16 CTAs of one site per thread per
// colour plane) in one cooperative launch of the resident kernel per span of
// sweeps (ResidentParams::pt): the sweeps, fused measurements, exchanges and
// records of k_ising_post's cycle without a kernel boundary.  Records go to
// the caller's arrays; the device ring is not used.  Returns 1 (and touches
// nothing) when the batch does not qualify, so the caller takes the graph path.
static int pt_resident(isg_ising* H, int64_t n_sweeps, int ee, int me, int32_t* tslot,
                       int64_t* bond, int64_t* mag, int64_t max_records, int64_t* n_records) {
    const int RT = H->replicas_total;
    if (!H->resident_pt || H->d_hist || H->records_made != H->records_done) return 1;
    uint32_t max_plane = 0;
    for (int s = 0; s < H->n_classes; ++s) max_plane = std::max(max_plane, H->P.cls[s].plane_sites);
    if (max_plane > 16u * kResidentThreads) return 1;
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, H->device);
    if (!coop) return 1;
    const void* kfun = H->dim == 3 ? (const void*)k_ising_resident<3>
                                   : (const void*)k_ising_resident<2>;
    if (cudaFuncSetAttribute(kfun, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
        cudaSuccess)
        cudaGetLastError();
    ResidentParams Q{};
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[2];
    int active = 0;
    if (!resident_config(H, cfg, attr, Q, kfun, max_plane, &active) || active < RT ||
        (1u << Q.log2_chunk) > (uint32_t)kResidentThreads)
        return 1;
    attr[1].id = cudaLaunchAttributeCooperative;
    attr[1].val.cooperative = 1;
    cfg.numAttrs = 2;
    const uint64_t k0 = H->ksample;
    const int64_t need = (int64_t)((k0 + (uint64_t)n_sweeps) / (uint64_t)me - k0 / (uint64_t)me);
    if (need > 0 && (!tslot || !bond || !mag || max_records < need))
        return fail(ISG_ERR_ARG, "isg_ising_pt_run: record arrays hold " +
                                     std::to_string(max_records) + " rows, " +
                                     std::to_string(need) + " needed");
    const int64_t span_max = (int64_t)1 << 16;
    const int64_t rows_max = span_max / me + 1;
    int rc = grow((void**)&H->d_srec, &H->srec_cap,
                  rows_max * RT * 2 * (int64_t)sizeof(unsigned long long));
    if (rc) return rc;
    rc = grow((void**)&H->d_srec_t, &H->srec_t_cap, rows_max * RT * (int64_t)sizeof(int32_t));
    if (rc) return rc;
    const int64_t scratch = (2 * (int64_t)RT + 2 * (int64_t)RT + 2) * 8;
    rc = grow((void**)&H->d_pt_scratch, &H->pt_scratch_cap, scratch);
    if (rc) return rc;
    unsigned long long* eacc = H->d_pt_scratch;
    double* ebuf = reinterpret_cast<double*>(H->d_pt_scratch + 2 * RT);
    unsigned int* bar = reinterpret_cast<unsigned int*>(H->d_pt_scratch + 4 * RT);
    int* err = reinterpret_cast<int*>(H->d_pt_scratch + 4 * RT + 1);
    Q.tables = H->d_thr;
    Q.sched = nullptr;
    Q.rec = H->d_srec;
    Q.measure_every = 0;
    Q.measure_phase = 0;
    Q.lattices = RT;
    for (int c = 0; c < kMaxClasses; ++c) {
        const int L = H->P.cls[c < H->n_classes ? c : 0].L;
        Q.div_half[c] = make_div((uint32_t)(L / 2));
        Q.div_L[c] = make_div((uint32_t)L);
    }
    Q.pt = 1;
    Q.ee = ee;
    Q.me = me;
    Q.rec_t = H->d_srec_t;
    Q.eacc = eacc;
    Q.ebuf = ebuf;
    Q.r2t = H->d_r2t;
    Q.t2r = H->d_t2r;
    Q.betas = H->d_betas;
    Q.ctrl = H->d_ctrl;
    Q.bar = bar;
    Q.err = err;
    Q.J = H->J;
    Q.h = H->h;
    Q.seed = H->seed;
    Q.n_classes = H->n_classes;
    int64_t done = 0, row = 0;
    std::vector<int32_t> tbuf;
    while (done < n_sweeps) {
        const int64_t n = std::min(span_max, n_sweeps - done);
        const uint64_t ks = H->ksample;
        const int64_t rows = (int64_t)((ks + (uint64_t)n) / (uint64_t)me - ks / (uint64_t)me);
        ISG_CK(cudaMemsetAsync(H->d_pt_scratch, 0, (size_t)scratch, H->stream));
        Q.sweep0 = H->gsweep;
        Q.ks0 = ks;
        Q.n_sweeps = n;
        cudaError_t e = H->dim == 3 ? cudaLaunchKernelEx(&cfg, k_ising_resident<3>, H->P, Q)
                                    : cudaLaunchKernelEx(&cfg, k_ising_resident<2>, H->P, Q);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (done == 0) return 1;  // this launch form is not available: graph path
            return cuda_fail(e, "cudaLaunchKernelEx(k_ising_resident, PT)");
        }
        launch_post(H, 0, 0, 0, 0, (int)n);  // device sweep counter
        H->gsweep += (uint64_t)n;
        H->ksample += (uint64_t)n;
        rc = check_launch("isg_ising_pt_run");
        if (rc) return rc;
        int herr = 0;
        ISG_CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, H->stream));
        ISG_CK(cudaStreamSynchronize(H->stream));
        if (herr)
            return fail(ISG_ERR_TIMEOUT, "isg_ising_pt_run: an exchange barrier wait gave up");
        if (rows > 0) {
            rc = copy_records(H, H->d_srec, rows, row, bond, mag);
            if (rc) return rc;
            ISG_CK(cudaMemcpy(tslot + (size_t)row * RT, H->d_srec_t,
                              (size_t)rows * RT * sizeof(int32_t), cudaMemcpyDeviceToHost));
            row += rows;
        }
        done += n;
    }
    if (n_records) *n_records = row;
    return ISG_OK;
}

static int schedule_sweeps(isg_ising* H, const double* temps, int64_t n_sweeps, int every,
                           int phase, int64_t* bond, int64_t* mag) {
    const int RT = H->replicas_total;
    int64_t row = 0;
    for (int64_t k = 0; k < n_sweeps; ++k) {
        if (temps && (k == 0 || temps[k] != temps[k - 1])) {
            int rc = all_slots_to(H, temps[k]);
            if (rc) return rc;
        }
        const bool meas = every > 0 && k % every == phase;
        if (meas)
            ISG_CK(cudaMemsetAsync(H->d_acc, 0, sizeof(unsigned long long) * 2 * RT, H->stream));
        launch_half(H, 0, 0, 0);
        launch_half(H, 1, 0, meas ? 1 : 0);
        launch_post(H, 0, 0, 0, 0, 1);
        H->gsweep += 1;
        int rc = check_launch("isg_ising_run_schedule");
        if (rc) return rc;
        if (meas) {
            rc = copy_records(H, H->d_acc, 1, row, bond, mag);
            if (rc) return rc;
            ++row;
        }
    }
    return ISG_OK;
}

}  // namespace isg

extern "C" {

int isg_ising_run_schedule(isg_ising* H, const double* temps, int64_t n_sweeps, int measure_every,
                           int measure_phase, int64_t* bond, int64_t* mag, int64_t max_rows,
                           int64_t* n_rows) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_run_schedule: NULL handle");
    if (!temps && !H->temps_set)
        return fail(ISG_ERR_STATE, "isg_ising_run_schedule: temperatures not set");
    if (n_sweeps < 0 || n_sweeps > ((int64_t)1 << 40) || measure_every < 0 ||
        (measure_every > 0 && (measure_phase < 0 || measure_phase >= measure_every)))
        return fail(ISG_ERR_ARG, "isg_ising_run_schedule: need n_sweeps >= 0, measure_every >= 0 "
                                 "and 0 <= measure_phase < measure_every");
    if (temps)
        for (int64_t k = 0; k < n_sweeps; ++k)
            if (!(temps[k] > 0.0) || !std::isfinite(temps[k]))
                return fail(ISG_ERR_ARG, "isg_ising_run_schedule: temperatures must be positive");
    const int64_t rows = count_rows(n_sweeps, measure_every, measure_phase);
    if (rows > 0 && (!bond || !mag || max_rows < rows))
        return fail(ISG_ERR_ARG, "isg_ising_run_schedule: record arrays hold " +
                                     std::to_string(max_rows) + " rows, " + std::to_string(rows) +
                                     " needed");
    if (n_rows) *n_rows = 0;
    if (n_sweeps == 0) return ISG_OK;
    cudaSetDevice(H->device);
    bool resident = true;
    for (int s = 0; s < H->n_classes; ++s)
        resident = resident && H->P.cls[s].plane_sites <= kResidentMaxPlane;
    const int every = rows > 0 ? measure_every : 0;
    int rc = ISG_OK;
    // the resident kernel reads schedule tables, not the slot tables, so the
    // slots take the final temperature up front (an upload after the launch
    // would wait for it); the sweep-by-sweep path sets them as it goes
    if (temps && resident) rc = all_slots_to(H, temps[n_sweeps - 1]);
    if (rc) return rc;
    rc = resident ? schedule_resident(H, temps, n_sweeps, every, measure_phase, bond, mag)
                  : schedule_sweeps(H, temps, n_sweeps, every, measure_phase, bond, mag);
    if (rc) return rc;
    if (temps) H->temps_set = true;
    if (n_rows) *n_rows = rows;
    return check_launch("isg_ising_run_schedule");
}

// ------------------------------------------------------------ histograms

static int hist_clear(isg_ising* H) {
    ISG_CK(cudaMemsetAsync(H->d_hist, 0, sizeof(unsigned long long) * 4 * H->hist_bins, H->stream));
    std::vector<int32_t> rng(2 * (size_t)H->replicas_total);
    for (size_t i = 0; i < rng.size(); i += 2) {
        rng[i] = INT32_MAX;
        rng[i + 1] = -1;
    }
    ISG_CK(cudaMemcpyAsync(H->d_hist_rng, rng.data(), sizeof(int32_t) * rng.size(),
                           cudaMemcpyHostToDevice, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

int isg_ising_hist_enable(isg_ising* H, int enable) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_hist_enable: NULL handle");
    cudaSetDevice(H->device);
    ISG_CK(cudaStreamSynchronize(H->stream));
    // cached graphs hold the record kernel's parameters: capture them again
    destroy_graph(H);
    if (!enable) {
        cudaFree(H->d_hist);
        cudaFree(H->d_hist_rng);
        H->d_hist = nullptr;
        H->d_hist_rng = nullptr;
        H->hist_bins = 0;
        H->Q.hist = nullptr;
        H->Q.hist_rng = nullptr;
        return ISG_OK;
    }
    if (H->d_hist) return hist_clear(H);
    int64_t total = 0;
    for (int s = 0; s < H->n_classes; ++s) {
        const int64_t L = H->sizes[s];
        const int64_t nsite = H->dim == 3 ? L * L * L : L * L;
        const int64_t dn = H->dim * nsite;
        if (dn > ((int64_t)1 << 33))
            return fail(ISG_ERR_UNSUPPORTED, "isg_ising_hist_enable: lattice too large");
        H->Q.hist_off[s] = (long long)total;
        H->Q.hist_dn[s] = (long long)dn;
        H->Q.hist_nsite[s] = (double)nsite;
        total += (int64_t)H->R * (dn / 2 + 1);
    }
    ISG_CK(cudaMalloc((void**)&H->d_hist, sizeof(unsigned long long) * 4 * total));
    cudaError_t e = cudaMalloc((void**)&H->d_hist_rng, sizeof(int32_t) * 2 * H->replicas_total);
    if (e != cudaSuccess) {
        cudaFree(H->d_hist);
        H->d_hist = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    H->hist_bins = total;
    H->Q.hist = H->d_hist;
    H->Q.hist_rng = H->d_hist_rng;
    return hist_clear(H);
}

int isg_ising_hist_reset(isg_ising* H) {
    if (!H) return fail(ISG_ERR_ARG, "isg_ising_hist_reset: NULL handle");
    if (!H->d_hist) return fail(ISG_ERR_STATE, "isg_ising_hist_reset: histograms are off");
    cudaSetDevice(H->device);
    return hist_clear(H);
}

int isg_ising_hist_range(isg_ising* H, int size_index, int slot, int64_t* bond_lo,
                         int64_t* n_bins) {
    if (!H || !bond_lo || !n_bins || size_index < 0 || size_index >= H->n_classes || slot < 0 ||
        slot >= H->R)
        return fail(ISG_ERR_ARG, "isg_ising_hist_range: bad argument");
    if (!H->d_hist) return fail(ISG_ERR_STATE, "isg_ising_hist_range: histograms are off");
    cudaSetDevice(H->device);
    int32_t rg[2];
    ISG_CK(cudaMemcpyAsync(rg, H->d_hist_rng + 2 * ((int64_t)size_index * H->R + slot),
                           sizeof(rg), cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    const int64_t dn = H->Q.hist_dn[size_index];
    if (rg[1] < rg[0]) {
        *bond_lo = -dn;
        *n_bins = 0;
    } else {
        *bond_lo = 4 * (int64_t)rg[0] - dn;
        *n_bins = (int64_t)rg[1] - rg[0] + 1;
    }
    return ISG_OK;
}

int isg_ising_hist_read(isg_ising* H, int size_index, int slot, int64_t bond_lo, int64_t n_bins,
                        uint64_t* out) {
    if (!H || size_index < 0 || size_index >= H->n_classes || slot < 0 || slot >= H->R ||
        n_bins < 0 || (n_bins > 0 && !out))
        return fail(ISG_ERR_ARG, "isg_ising_hist_read: bad argument");
    if (!H->d_hist) return fail(ISG_ERR_STATE, "isg_ising_hist_read: histograms are off");
    const int64_t dn = H->Q.hist_dn[size_index];
    if (((bond_lo + dn) & 3) != 0 || bond_lo < -dn || bond_lo + 4 * (n_bins - 1) > dn)
        return fail(ISG_ERR_ARG, "isg_ising_hist_read: bins must lie in [-dN, dN] with "
                                 "bond_lo + dN a multiple of 4");
    if (n_bins == 0) return ISG_OK;
    cudaSetDevice(H->device);
    const int64_t row = H->Q.hist_off[size_index] + (int64_t)slot * (dn / 2 + 1) + (bond_lo + dn) / 4;
    ISG_CK(cudaMemcpyAsync(out, H->d_hist + 4 * row, sizeof(unsigned long long) * 4 * n_bins,
                           cudaMemcpyDeviceToHost, H->stream));
    ISG_CK(cudaStreamSynchronize(H->stream));
    return ISG_OK;
}

}  // extern "C"
