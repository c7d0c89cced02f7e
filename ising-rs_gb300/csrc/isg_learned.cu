// isg_learned.cu — learned autoregressive proposal for Ising configurations.
//
// No reference counterpart (faulknco/ising-rs has only a CNN phase classifier,
// analysis/ml_phase.ipynb).  A masked-convolution autoregressive network over
// the lattice in raster order (row-major, H rows of W sites; a cubic L^3
// lattice is the H = L^2, W = L image of its z-y rows) gives
//   q(s) = prod_i sigma(s_i * logit_i(s_<i)),
// symmetrised as q_sym(s) = (q(s) + q(-s)) / 2.  Proposals drawn from q_sym are
// accepted by an exact independence Metropolis-Hastings test; log q_sym comes
// from the same deterministic kernel in sampling and in scoring mode, so the
// chain targets exp(-beta E) exactly.
//
// Network: layer 0 is a 3x3 mask-A convolution (taps above and to the left,
// excluding the centre) from 1 to C channels; layers 1..D-2 are 3x3 mask-B
// convolutions (mask A plus the centre) C -> C; layer D-1 is mask B, C -> 1
// (the logit).  Hidden layers use ReLU; zero padding at the lattice edges.
// Weights are stored in BF16 and all products accumulate in FP32; training
// keeps FP32 master weights (Adam) and refreshes the BF16 copy every step.
// Sampling and scoring run on the tensor cores (k_ar_mma, BF16 activations
// between layers) when the network's activation rings fit in shared memory,
// else on the CUDA cores (k_ar_run, FP32 activations).  Scoring given
// configurations uses k_ar_score (all positions of a layer at once) when its
// buffers fit; it repeats k_ar_mma's arithmetic element by element, so a
// proposal's log q is the same whichever kernel computes it.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {
namespace {

constexpr int kC = 32;         // channels
constexpr int kMaxLayers = 8;
__host__ __device__ __forceinline__ int tap_dx(int t) { return t < 3 ? t - 1 : (t == 3 ? -1 : 0); }
constexpr uint32_t kTagLearn = 0x06u;

// Weight layout per layer l: w[tap][cin][cout] (taps 0..3 for layer 0, 0..4
// for a 3D network's layer 0 and for the other layers), then bias[cout].
// cin = 1 for layer 0, cout = 1 for the last layer.
struct NetShape {
    int D;                       // layers
    int zrow;                    // rows per z-plane of a 3D lattice's raster (0: 2D)
    int cin[kMaxLayers], cout[kMaxLayers], taps[kMaxLayers];
    int woff[kMaxLayers];        // offset of layer weights
    int boff[kMaxLayers];        // offset of layer bias
    int total;
};

NetShape make_shape(int D, int zrow) {
    NetShape s{};
    s.D = D;
    s.zrow = zrow;
    int off = 0;
    for (int l = 0; l < D; ++l) {
        s.cin[l] = l == 0 ? 1 : kC;
        s.cout[l] = l == D - 1 ? 1 : kC;
        s.taps[l] = l == 0 ? (zrow > 0 ? 5 : 4) : 5;
        s.woff[l] = off;
        off += s.taps[l] * s.cin[l] * s.cout[l];
        s.boff[l] = off;
        off += s.cout[l];
    }
    s.total = off;
    return s;
}

// Row offset of tap t of layer l: taps 0..2 look one row back, tap 3 along
// the row; tap 4 is the centre for layers >= 1 and, for layer 0 of a 3D
// network (whose raster is the L^2 x L image of its z-y rows), the site one
// z-plane back: zrow rows up, same x.  In raster order that site precedes the
// current one, so the mask stays autoregressive.
__host__ __device__ __forceinline__ int tap_dy(const NetShape& S, int l, int t) {
    return (l == 0 && t == 4) ? -S.zrow : (t < 3 ? -1 : 0);
}
// Rows of layer l's input that its taps reach back, staged by k_tf_wgrad.
__host__ __device__ __forceinline__ int wg_halo(const NetShape& S, int l, int W) {
    return (l == 0 && S.zrow > 0 && S.zrow * W > W + 1) ? S.zrow * W : W + 1;
}

__device__ __forceinline__ float bf(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

__device__ __forceinline__ float log_sigmoid(float z) {
    // log(1 / (1 + e^-z)) computed stably
    return z >= 0.f ? -log1pf(__expf(-z)) : z - log1pf(__expf(z));
}

// -------------------------------------------------------------- AR kernel
// Sampling / scoring, G configurations per block, positions in raster order.
// Activation rings hold the last W+2 positions of every layer output.
// mode 0: sample s (Philox: uid = proposal index, c1 = position, step),
//         write s and log q(s); mode 1: score the given s (log q only).
// If `flip` is set, the configuration scored is -s.
template <int G>
__global__ void __launch_bounds__(G * kC)
    k_ar_run(const __nv_bfloat16* __restrict__ w, NetShape S, int H, int W, int mode, int flip,
             int8_t* __restrict__ spins, float* __restrict__ logq, int n_cfg, uint64_t seed,
             uint64_t step) {
    extern __shared__ float sm[];
    const int ring = W + 2;
    // layout: rings for layer outputs 0..D-2: [(D-1)][ring][G][kC]; spins [G][H*W] int8
    float* rings = sm;
    int8_t* sp = reinterpret_cast<int8_t*>(sm + (size_t)(S.D - 1) * ring * G * kC);
    const int g = threadIdx.x / kC;   // configuration within the block
    const int c = threadIdx.x % kC;   // output channel handled
    const int cfg = blockIdx.x * G + g;
    const bool live = cfg < n_cfg;
    const int HW = H * W;
    if (mode == 1) {
        for (int i = threadIdx.x; i < G * HW; i += blockDim.x) {
            const int gg = i / HW, p = i - gg * HW;
            const int cc = blockIdx.x * G + gg;
            int8_t v = cc < n_cfg ? spins[(size_t)cc * HW + p] : (int8_t)1;
            sp[i] = flip ? (int8_t)-v : v;
        }
    }
    __syncthreads();
    float lq = 0.f;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t c3 = counter_word3(kTagLearn, 0, step);
    for (int p = 0; p < HW; ++p) {
        const int y = p / W, x = p - y * W;
        const int slot = p % ring;
        for (int l = 0; l < S.D; ++l) {
            const int taps = S.taps[l];
            const bool last = l == S.D - 1;
            float acc = 0.f;
            if (!last || c == 0) {
                const int co = last ? 0 : c;
                acc = bf(w, S.boff[l] + co);
                for (int t = 0; t < taps; ++t) {
                    const int yy = y + tap_dy(S, l, t), xx = x + tap_dx(t);
                    if (yy < 0 || xx < 0 || xx >= W) continue;
                    const int q = yy * W + xx;
                    const __nv_bfloat16* wt = w + S.woff[l] + (t * S.cin[l]) * S.cout[l] + co;
                    if (l == 0) {
                        acc = fmaf(bf(wt, 0), (float)sp[g * HW + q], acc);
                    } else {
                        const float* a = rings + ((size_t)(l - 1) * ring + (q % ring)) * G * kC +
                                         g * kC;
                        for (int ci = 0; ci < kC; ++ci) acc = fmaf(bf(wt, ci * S.cout[l]), a[ci], acc);
                    }
                }
            }
            if (!last) {
                rings[((size_t)l * ring + slot) * G * kC + g * kC + c] = fmaxf(acc, 0.f);
                __syncthreads();
            } else if (c == 0 && live) {
                int8_t s;
                if (mode == 0) {
                    const U4 u = philox10((uint32_t)cfg, (uint32_t)p, (uint32_t)step, c3, k0, k1);
                    // P(s = +1) = sigmoid(logit)
                    const float pr = 1.0f / (1.0f + __expf(-acc));
                    s = uniform24(u.x) < pr ? (int8_t)1 : (int8_t)-1;
                    sp[g * HW + p] = s;
                } else {
                    s = sp[g * HW + p];
                }
                lq += log_sigmoid((float)s * acc);
            }
        }
        __syncthreads();  // the sampled spin is visible before the next position
    }
    if (c == 0 && live) {
        logq[cfg] = lq;
        if (mode == 0)
            for (int p = 0; p < HW; ++p) spins[(size_t)cfg * HW + p] = sp[g * HW + p];
    }
}

// -------------------------------------------------------------- training
// Teacher-forced forward of one layer for a batch: out[b][p][co] (pre-ReLU
// stored in z, post in a) from in[b][p][ci].
__global__ void k_tf_layer(const __nv_bfloat16* __restrict__ w, NetShape S, int l, int H, int W,
                           int B, const float* __restrict__ in, float* __restrict__ z,
                           float* __restrict__ a) {
    const int HW = H * W;
    const int cin = S.cin[l], cout = S.cout[l], taps = S.taps[l];
    const int64_t total = (int64_t)B * HW * cout;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int co = (int)(i % cout);
        const int64_t bp = i / cout;
        const int p = (int)(bp % HW);
        const int64_t b = bp / HW;
        const int y = p / W, x = p - y * W;
        float acc = bf(w, S.boff[l] + co);
        for (int t = 0; t < taps; ++t) {
            const int yy = y + tap_dy(S, l, t), xx = x + tap_dx(t);
            if (yy < 0 || xx < 0 || xx >= W) continue;
            const float* src = in + (b * HW + yy * W + xx) * cin;
            const __nv_bfloat16* wt = w + S.woff[l] + (t * cin) * cout + co;
            for (int ci = 0; ci < cin; ++ci) acc = fmaf(bf(wt, ci * cout), src[ci], acc);
        }
        z[i] = acc;
        if (a) a[i] = fmaxf(acc, 0.f);
    }
}

// Output gradient: loss = -(1/B) sum_b log q(s_b); dL/dlogit = -(1/B) s sigma(-s logit).
// Also returns per-config log q (sum of log sigmoid) in lq.
__global__ void k_tf_out_grad(const float* __restrict__ logit, const float* __restrict__ sx,
                              int HW, int B, float* __restrict__ dz, float* __restrict__ lq) {
    const int b = blockIdx.x;
    float acc = 0.f;
    for (int p = threadIdx.x; p < HW; p += blockDim.x) {
        const float s = sx[(int64_t)b * HW + p];
        const float zl = logit[(int64_t)b * HW + p];
        const float sg = 1.0f / (1.0f + __expf(s * zl));  // sigma(-s z)
        dz[(int64_t)b * HW + p] = -s * sg / (float)B;
        acc += log_sigmoid(s * zl);
    }
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) lq[b] = red[0];
}

// Input gradient of layer l: d_in[b][p][ci] = sum_t sum_co w[t][ci][co] dz[b][p - off_t][co],
// multiplied by relu'(z_in) when the input is a hidden activation.
__global__ void k_tf_dgrad(const __nv_bfloat16* __restrict__ w, NetShape S, int l, int H, int W,
                           int B, const float* __restrict__ dz, const float* __restrict__ zin,
                           float* __restrict__ din) {
    const int HW = H * W;
    const int cin = S.cin[l], cout = S.cout[l], taps = S.taps[l];
    const int64_t total = (int64_t)B * HW * cin;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int64_t bp = i / cin;
        const int p = (int)(bp % HW);
        const int64_t b = bp / HW;
        const int y = p / W, x = p - y * W;
        float acc = 0.f;
        for (int t = 0; t < taps; ++t) {
            // output position q with q + off_t = p
            const int yy = y - tap_dy(S, l, t), xx = x - tap_dx(t);
            if (yy >= H || xx < 0 || xx >= W) continue;
            const float* g = dz + (b * HW + yy * W + xx) * cout;
            const __nv_bfloat16* wt = w + S.woff[l] + (t * cin + ci) * cout;
            for (int co = 0; co < cout; ++co) acc = fmaf(bf(wt, co), g[co], acc);
        }
        if (zin) acc = zin[i] > 0.f ? acc : 0.f;
        din[i] = acc;
    }
}

// Weight and bias gradient partials of layer l: block k covers positions
// [k*chunk, (k+1)*chunk) of the flattened batch; thread j accumulates weights
// j, j + blockDim, ...  (tap, ci, co), plus the biases.
// Weight and bias gradient partials of layer l over one chunk of `chunk`
// flattened positions bp = b*HW + p (one block per chunk): the chunk's output
// gradients and the input rows its taps reach (bp - W - 1 .. bp) are staged in
// shared memory with a per-position tap-validity mask, then every thread
// accumulates its weights over the chunk.  part[block][j], j = weights then
// biases, summed in block order by k_sum_parts.
__global__ void k_tf_wgrad(NetShape S, int l, int H, int W, int B, const float* __restrict__ in,
                           const float* __restrict__ dz, int chunk, float* __restrict__ part) {
    extern __shared__ float wg_sm[];
    const int HW = H * W;
    const int cin = S.cin[l], cout = S.cout[l], taps = S.taps[l];
    const int nw = taps * cin * cout + cout;
    const int64_t n = (int64_t)B * HW;
    const int64_t start = (int64_t)blockIdx.x * chunk;
    const int cnt = (int)(start + chunk < n ? chunk : n - start);
    const int halo = wg_halo(S, l, W);
    float* s_dz = wg_sm;                              // [chunk][cout]
    float* s_in = s_dz + (size_t)chunk * cout;        // [halo + chunk][cin]
    unsigned char* s_ok = reinterpret_cast<unsigned char*>(s_in + (size_t)(halo + chunk) * cin);
    for (int i = threadIdx.x; i < cnt * cout; i += blockDim.x) s_dz[i] = dz[start * cout + i];
    for (int i = threadIdx.x; i < (halo + cnt) * cin; i += blockDim.x) {
        const int64_t row = start - halo + i / cin;
        s_in[i] = row >= 0 ? in[row * cin + i % cin] : 0.f;
    }
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
        const int p = (int)((start + q) % HW);
        const int y = p / W, x = p - y * W;
        unsigned char m = 0;
        for (int t = 0; t < taps; ++t) {
            const int yy = y + tap_dy(S, l, t), xx = x + tap_dx(t);
            if (yy >= 0 && xx >= 0 && xx < W) m |= (unsigned char)(1u << t);
        }
        s_ok[q] = m;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nw; j += blockDim.x) {
        float acc = 0.f;
        if (j < taps * cin * cout) {
            const int co = j % cout;
            const int ci = (j / cout) % cin;
            const int t = j / (cout * cin);
            const int off = halo + tap_dy(S, l, t) * W + tap_dx(t);  // s_in row of q's tap
            const unsigned char bit = (unsigned char)(1u << t);
            for (int q = 0; q < cnt; ++q)
                if (s_ok[q] & bit) acc = fmaf(s_in[(q + off) * cin + ci], s_dz[q * cout + co], acc);
        } else {
            const int co = j - taps * cin * cout;
            for (int q = 0; q < cnt; ++q) acc += s_dz[q * cout + co];
        }
        part[(int64_t)blockIdx.x * nw + j] = acc;
    }
}

// -------------------------------------------- training on the tensor cores
// The convolutions of the layers with 32 input channels (layers 1..D-1) as
// implicit GEMMs on mma.sync m16n8k8 with TF32 operands and FP32
// accumulation.  An FP32 operand x is split into hi = tf32(x) and lo =
// tf32(x - hi), and a product takes the MMAs a_lo b + a_hi b (the BF16
// weights are exact in TF32), or a_lo b_hi + a_hi b_lo + a_hi b_hi for the
// weight gradient, so the sums keep FP32 accuracy to about 1e-6 relative.  Rows (16 per warp) are positions m = b HW + p of the
// flattened batch; a block stages the rows its taps reach (rows padded to
// 36 words, so a warp's fragment loads hit 32 different banks) and the layer's
// weights (k = tap * 32 + channel, rows padded to 40 words, likewise).  Layer
// 0 (one input channel) stays on the CUDA cores.
constexpr int kTcTile = 128;   // positions per block tile (8 warps x 16)
constexpr int kTcRow = 36;     // staged words per position row
constexpr int kTcWRow = 40;    // staged words per weight row
constexpr int kTcChunk = 512;  // positions per block of the weight gradient

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
// hi / lo TF32 parts of an FP32 value held as its bit pattern
__device__ __forceinline__ void split_tf32(uint32_t x, uint32_t& hi, uint32_t& lo) {
    const float f = __uint_as_float(x);
    hi = to_tf32(f);
    lo = to_tf32(f - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float* d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
// Tap t of layer l >= 1 at position p: its offset in the flattened batch and
// whether it lies inside the lattice.
__device__ __forceinline__ bool tc_tap(const NetShape& S, int l, int t, int p, int W, int& off) {
    const int dy = tap_dy(S, l, t), dx = tap_dx(t);
    const int y = p / W, x = p - y * W;
    off = dy * W + dx;
    return y + dy >= 0 && x + dx >= 0 && x + dx < W;
}
__host__ __device__ inline size_t tc_fwd_smem(int W) {
    return sizeof(uint32_t) * ((size_t)5 * kC * kTcWRow + (size_t)(W + 1 + kTcTile + 1) * kTcRow);
}
__host__ __device__ inline size_t tc_wgrad_smem(int W) {
    return sizeof(uint32_t) * ((size_t)(W + 1 + kTcChunk) * kTcRow + (size_t)kTcChunk * kTcWRow) +
           (size_t)kTcChunk;
}

// Forward of layer l >= 1: z[m][co] = bias[co] + sum_t sum_ci w[t][ci][co]
// in[m + off_t][ci] (taps outside the lattice add nothing), a = relu(z) for a
// hidden layer.  cout = 32, or 1 for the last layer.
__global__ void __launch_bounds__(256) k_tc_fwd(const __nv_bfloat16* __restrict__ w, NetShape S,
                                                int l, int H, int W, int B,
                                                const float* __restrict__ in,
                                                float* __restrict__ z, float* __restrict__ a) {
    extern __shared__ uint32_t tsm[];
    const int cout = S.cout[l], nt = cout == 1 ? 1 : 4;
    const int HW = H * W, halo = W + 1;
    const int64_t M = (int64_t)B * HW;
    uint32_t* s_w = tsm;                                  // [160][kTcWRow]
    uint32_t* s_in = s_w + 5 * kC * kTcWRow;              // [halo + tile + 1][kTcRow]
    const uint32_t* zrow = s_in + (size_t)(halo + kTcTile) * kTcRow;
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5, g = lane >> 2, q = lane & 3;
    for (int i = tid; i < 5 * kC * kTcWRow; i += blockDim.x) {
        const int k = i / kTcWRow, n = i - k * kTcWRow;
        s_w[i] = n < cout ? to_tf32(bf(w, S.woff[l] + k * cout + n)) : 0u;
    }
    for (int i = tid; i < kTcRow; i += blockDim.x) s_in[(size_t)(halo + kTcTile) * kTcRow + i] = 0u;
    for (int64_t m0 = (int64_t)blockIdx.x * kTcTile; m0 < M; m0 += (int64_t)gridDim.x * kTcTile) {
        __syncthreads();  // the previous tile's reads are done
        for (int i = tid; i < (halo + kTcTile) * kC; i += blockDim.x) {
            const int r = i >> 5, c = i & 31;
            const int64_t mm = m0 - halo + r;
            s_in[r * kTcRow + c] = (mm >= 0 && mm < M) ? __float_as_uint(in[mm * kC + c]) : 0u;
        }
        __syncthreads();
        const int rA = 16 * wp + g, rB = rA + 8;  // rows of the tile
        const int64_t mA = m0 + rA, mB = m0 + rB;
        const int pA = (int)(mA % HW), pB = (int)(mB % HW);
        float acc[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            int offA, offB;
            const bool vA = tc_tap(S, l, t, pA, W, offA) && mA < M;
            const bool vB = tc_tap(S, l, t, pB, W, offB) && mB < M;
            const uint32_t* ra = vA ? s_in + (size_t)(halo + rA + offA) * kTcRow : zrow;
            const uint32_t* rb = vB ? s_in + (size_t)(halo + rB + offB) * kTcRow : zrow;
#pragma unroll
            for (int cb = 0; cb < 4; ++cb) {
                uint32_t h0, h1, h2, h3, l0, l1, l2, l3;
                split_tf32(ra[8 * cb + q], h0, l0);
                split_tf32(rb[8 * cb + q], h1, l1);
                split_tf32(ra[8 * cb + q + 4], h2, l2);
                split_tf32(rb[8 * cb + q + 4], h3, l3);
                const uint32_t* wk = s_w + (size_t)((t * 4 + cb) * 8 + q) * kTcWRow;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j < nt) {
                        const uint32_t b0 = wk[8 * j + g], b1 = wk[4 * kTcWRow + 8 * j + g];
                        mma_tf32(acc[j], l0, l1, l2, l3, b0, b1);
                        mma_tf32(acc[j], h0, h1, h2, h3, b0, b1);
                    }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (j >= nt) break;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int n = 8 * j + 2 * q + (e & 1);
                const int64_t m = e < 2 ? mA : mB;
                if (n < cout && m < M) {
                    const float v = acc[j][e] + bf(w, S.boff[l] + n);
                    z[m * cout + n] = v;
                    if (a) a[m * cout + n] = fmaxf(v, 0.f);
                }
            }
        }
    }
}

// Input gradient of a hidden layer l >= 1 (cin = cout = 32):
// din[m][ci] = relu'(zin[m][ci]) sum_t sum_co w[t][ci][co] dz[m - off_t][co],
// where the position m - off_t is the one whose tap t reads m.
__global__ void __launch_bounds__(256) k_tc_dgrad(const __nv_bfloat16* __restrict__ w, NetShape S,
                                                  int l, int H, int W, int B,
                                                  const float* __restrict__ dz,
                                                  const float* __restrict__ zin,
                                                  float* __restrict__ din) {
    extern __shared__ uint32_t tsm[];
    const int HW = H * W, halo = W + 1;
    const int64_t M = (int64_t)B * HW;
    uint32_t* s_w = tsm;                      // [k = t*32 + co][n = ci]
    uint32_t* s_dz = s_w + 5 * kC * kTcWRow;  // rows m0 .. m0 + tile + halo
    const uint32_t* zrow = s_dz + (size_t)(halo + kTcTile) * kTcRow;
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5, g = lane >> 2, q = lane & 3;
    for (int i = tid; i < 5 * kC * kTcWRow; i += blockDim.x) {
        const int k = i / kTcWRow, n = i - k * kTcWRow;
        const int t = k >> 5, co = k & 31;
        s_w[i] = n < kC ? to_tf32(bf(w, S.woff[l] + (t * kC + n) * kC + co)) : 0u;
    }
    for (int i = tid; i < kTcRow; i += blockDim.x) s_dz[(size_t)(halo + kTcTile) * kTcRow + i] = 0u;
    for (int64_t m0 = (int64_t)blockIdx.x * kTcTile; m0 < M; m0 += (int64_t)gridDim.x * kTcTile) {
        __syncthreads();
        for (int i = tid; i < (halo + kTcTile) * kC; i += blockDim.x) {
            const int r = i >> 5, c = i & 31;
            const int64_t mm = m0 + r;
            s_dz[r * kTcRow + c] = mm < M ? __float_as_uint(dz[mm * kC + c]) : 0u;
        }
        __syncthreads();
        const int rA = 16 * wp + g, rB = rA + 8;
        const int64_t mA = m0 + rA, mB = m0 + rB;
        const int pA = (int)(mA % HW), pB = (int)(mB % HW);
        float acc[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            // the position whose tap t reads p: p - off_t, inside the lattice
            const int dy = tap_dy(S, l, t), dx = tap_dx(t), off = dy * W + dx;
            const int yA = pA / W, xA = pA - yA * W, yB = pB / W, xB = pB - yB * W;
            const bool vA = mA < M && yA - dy < H && xA - dx >= 0 && xA - dx < W;
            const bool vB = mB < M && yB - dy < H && xB - dx >= 0 && xB - dx < W;
            const uint32_t* ra = vA ? s_dz + (size_t)(rA - off) * kTcRow : zrow;
            const uint32_t* rb = vB ? s_dz + (size_t)(rB - off) * kTcRow : zrow;
#pragma unroll
            for (int cb = 0; cb < 4; ++cb) {
                uint32_t h0, h1, h2, h3, l0, l1, l2, l3;
                split_tf32(ra[8 * cb + q], h0, l0);
                split_tf32(rb[8 * cb + q], h1, l1);
                split_tf32(ra[8 * cb + q + 4], h2, l2);
                split_tf32(rb[8 * cb + q + 4], h3, l3);
                const uint32_t* wk = s_w + (size_t)((t * 4 + cb) * 8 + q) * kTcWRow;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t b0 = wk[8 * j + g], b1 = wk[4 * kTcWRow + 8 * j + g];
                    mma_tf32(acc[j], l0, l1, l2, l3, b0, b1);
                    mma_tf32(acc[j], h0, h1, h2, h3, b0, b1);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int n = 8 * j + 2 * q + (e & 1);
                const int64_t m = e < 2 ? mA : mB;
                if (m < M) din[m * kC + n] = zin[m * kC + n] > 0.f ? acc[j][e] : 0.f;
            }
    }
}

// Weight and bias gradient partials of layer l >= 1 over one chunk of
// kTcChunk positions (one block of 10 warps per chunk):
// part[block][(t*32 + ci)*cout + co] = sum_m [tap t of m inside] in[m + off_t][ci] dz[m][co],
// then the cout bias sums.  Warp r computes rows (t, ci) = 16 r .. 16 r + 15.
__global__ void __launch_bounds__(320) k_tc_wgrad(NetShape S, int l, int H, int W, int B,
                                                  const float* __restrict__ in,
                                                  const float* __restrict__ dz,
                                                  float* __restrict__ part) {
    extern __shared__ uint32_t tsm[];
    const int cout = S.cout[l], nt = cout == 1 ? 1 : 4;
    const int HW = H * W, halo = W + 1;
    const int64_t M = (int64_t)B * HW;
    const int nw = 5 * kC * cout + cout;
    const int64_t m0 = (int64_t)blockIdx.x * kTcChunk;
    uint32_t* s_in = tsm;                                          // [halo + chunk][kTcRow]
    uint32_t* s_dz = s_in + (size_t)(halo + kTcChunk) * kTcRow;    // [chunk][kTcWRow]
    unsigned char* s_ok = reinterpret_cast<unsigned char*>(s_dz + (size_t)kTcChunk * kTcWRow);
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5, g = lane >> 2, q = lane & 3;
    for (int i = tid; i < (halo + kTcChunk) * kC; i += blockDim.x) {
        const int r = i >> 5, c = i & 31;
        const int64_t mm = m0 - halo + r;
        s_in[r * kTcRow + c] = (mm >= 0 && mm < M) ? __float_as_uint(in[mm * kC + c]) : 0u;
    }
    for (int i = tid; i < kTcChunk * kTcWRow; i += blockDim.x) {
        const int r = i / kTcWRow, c = i - r * kTcWRow;
        const int64_t mm = m0 + r;
        s_dz[i] = (c < cout && mm < M) ? __float_as_uint(dz[mm * cout + c]) : 0u;
    }
    for (int r = tid; r < kTcChunk; r += blockDim.x) {
        const int64_t mm = m0 + r;
        unsigned char bits = 0;
        if (mm < M) {
            const int p = (int)(mm % HW);
            for (int t = 0; t < 5; ++t) {
                int off;
                if (tc_tap(S, l, t, p, W, off)) bits |= (unsigned char)(1u << t);
            }
        }
        s_ok[r] = bits;
    }
    __syncthreads();
    // warp wp: tap t = wp / 2, channels ci0 .. ci0 + 15
    const int t = wp >> 1, ci0 = (wp & 1) * 16;
    const int off = tap_dy(S, l, t) * W + tap_dx(t);
    const unsigned char bit = (unsigned char)(1u << t);
    float acc[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
    for (int kb = 0; kb < kTcChunk; kb += 8) {
        // A[row = ci][col = position]: in[m + off][ci] where tap t of m is inside
        const int c0 = kb + q, c1 = c0 + 4;
        const bool v0 = (s_ok[c0] & bit) != 0, v1 = (s_ok[c1] & bit) != 0;
        const uint32_t* r0 = s_in + (size_t)(halo + c0 + off) * kTcRow + ci0;
        const uint32_t* r1 = s_in + (size_t)(halo + c1 + off) * kTcRow + ci0;
        uint32_t h0, h1, h2, h3, l0, l1, l2, l3;
        split_tf32(v0 ? r0[g] : 0u, h0, l0);
        split_tf32(v0 ? r0[g + 8] : 0u, h1, l1);
        split_tf32(v1 ? r1[g] : 0u, h2, l2);
        split_tf32(v1 ? r1[g + 8] : 0u, h3, l3);
        const uint32_t* bk = s_dz + (size_t)(kb + q) * kTcWRow;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (j < nt) {
                uint32_t bh0, bl0, bh1, bl1;
                split_tf32(bk[8 * j + g], bh0, bl0);
                split_tf32(bk[4 * kTcWRow + 8 * j + g], bh1, bl1);
                mma_tf32(acc[j], l0, l1, l2, l3, bh0, bh1);
                mma_tf32(acc[j], h0, h1, h2, h3, bl0, bl1);
                mma_tf32(acc[j], h0, h1, h2, h3, bh0, bh1);
            }
    }
    float* pb = part + (int64_t)blockIdx.x * nw;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (j >= nt) break;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int ci = ci0 + g + (e < 2 ? 0 : 8);
            const int co = 8 * j + 2 * q + (e & 1);
            if (co < cout) pb[(t * kC + ci) * cout + co] = acc[j][e];
        }
    }
    // bias partials: sum of dz over the chunk, in position order
    for (int co = tid; co < cout; co += blockDim.x) {
        float sacc = 0.f;
        for (int r = 0; r < kTcChunk; ++r) {
            const int64_t mm = m0 + r;
            if (mm < M) sacc += dz[mm * cout + co];
        }
        pb[5 * kC * cout + co] = sacc;
    }
}

__global__ void k_sum_parts(const float* __restrict__ part, int nparts, int nw,
                            float* __restrict__ grad) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nw) return;
    float acc = 0.f;
    for (int k = 0; k < nparts; ++k) acc += part[(int64_t)k * nw + j];
    grad[j] = acc;
}

__global__ void k_adam(float* __restrict__ master, __nv_bfloat16* __restrict__ wbf,
                       const float* __restrict__ grad, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float v = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = v;
    const float upd = lr * (a / bc1) / (sqrtf(v / bc2) + eps);
    master[i] -= upd;
    wbf[i] = __float2bfloat16(master[i]);
}

// -------------------------------------------------------------- chain
// Exact energy pieces of natural-layout configurations: bond sum over the
// forward bonds of a periodic L^dim lattice and the magnetisation.
__global__ void k_cfg_energy(const int8_t* __restrict__ s, int L, int dim, int n_cfg,
                             long long* __restrict__ bond, long long* __restrict__ mag) {
    const int b = blockIdx.x;
    if (b >= n_cfg) return;
    const int n = dim == 3 ? L * L * L : L * L;
    const int8_t* c = s + (int64_t)b * n;
    long long bb = 0, mm = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = i % L, y = (i / L) % L, z = dim == 3 ? i / (L * L) : 0;
        const int v = c[i];
        mm += v;
        bb += v * c[(i - x) + (x + 1) % L];
        bb += v * c[(dim == 3 ? z * L * L : 0) + ((y + 1) % L) * L + x];
        if (dim == 3) bb += v * c[((z + 1) % L) * L * L + y * L + x];
    }
    __shared__ long long rb[256], rm[256];
    rb[threadIdx.x] = bb;
    rm[threadIdx.x] = mm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            rb[threadIdx.x] += rb[threadIdx.x + o];
            rm[threadIdx.x] += rm[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        bond[b] = rb[0];
        mag[b] = rm[0];
    }
}

// Independence Metropolis-Hastings over K proposals.  With
// A(s) = -beta E(s) - log q_sym(s), proposal y is accepted from state x iff
// log u < A(y) - A(x) (the test u < min(1, pi(y) q(x) / (pi(x) q(y)))).
// k_imh_prep evaluates A and log u for every proposal in parallel; k_imh_scan
// runs the sequential chain (one thread, one compare per proposal).
__global__ void k_imh_prep(const long long* __restrict__ bond, const float* __restrict__ lq_a,
                           const float* __restrict__ lq_b, int K, double beta, double J,
                           double* __restrict__ A, double* __restrict__ logu, uint64_t seed,
                           uint64_t step) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const double la = lq_a[k], lb = lq_b[k];
    const double mx = la > lb ? la : lb;
    const double lsym = mx + log(0.5 * (exp(la - mx) + exp(lb - mx)));
    const double E = -J * (double)bond[k];
    A[k] = -beta * E - lsym;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const U4 u = philox10(0xFFFFFFF0u, (uint32_t)k, (uint32_t)step, counter_word3(kTagLearn, 1, step),
                          k0, k1);
    logu[k] = log(uniform53(u.x, u.y));
}

// state = (bond, mag, index of the current configuration, -1 = unchanged);
// ax = A of the current state.  mrec[k] = |M| after proposal k.
__global__ void k_imh_scan(const long long* __restrict__ bond, const long long* __restrict__ mag,
                           const double* __restrict__ A, const double* __restrict__ logu, int K,
                           long long* __restrict__ state, double* __restrict__ ax,
                           long long* __restrict__ mrec, long long* __restrict__ brec,
                           long long* __restrict__ accepted) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long bx = state[0], mx = state[1], ix = -1;
    double a = *ax;
    long long acc = 0;
    for (int k = 0; k < K; ++k) {
        const double ak = A[k];
        if (logu[k] < ak - a) {
            a = ak;
            bx = bond[k];
            mx = mag[k];
            ix = k;
            ++acc;
        }
        mrec[k] = mx < 0 ? -mx : mx;
        if (brec) brec[k] = bx;
    }
    state[0] = bx;
    state[1] = mx;
    state[2] = ix;
    *ax = a;
    *accepted += acc;
}

// If the chain ended on proposal state[2] >= 0, copy it into the current
// configuration.
__global__ void k_adopt(const int8_t* __restrict__ props, const long long* __restrict__ state,
                        int8_t* __restrict__ cur, int n) {
    const long long j = state[2];
    if (j < 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        cur[i] = props[j * (long long)n + i];
}

// -------------------------------------------------- tensor-core AR kernel
// The same network and random stream as k_ar_run, 16 configurations per CTA:
// at every raster position each hidden layer is one [16 configs x 160] x
// [160 x 32] product (5 taps x 32 input channels) on the tensor cores
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation), fed by ldmatrix from
// the activation rings; layer 0 (1 input channel) runs on the CUDA cores.
// Rings hold the last W+2 positions of every hidden layer's BF16 output, 64 B
// per configuration row with the 16-byte chunks XOR-swizzled by (row >> 1) & 3
// so that ldmatrix reads are conflict-free; the transposed weights (rows =
// output channel, 160 k values, padded to 336 B rows) are staged once per CTA.
// An M >= 64 tcgen05 tile would need >= 680 KB of ring history per CTA, so the
// warp-level tensor instructions are the ones this per-position chain fits.
constexpr int kMmaRows = 16;
constexpr int kBtRow = 168;  // bf16 per transposed weight row (160 + 8 pad)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3,
                                        uint32_t addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
// byte offset of (row, 16-byte chunk) in a ring slot tile of 16 rows x 64 B
__device__ __forceinline__ uint32_t ring_off(int row, int chunk) {
    return (uint32_t)(row * 64 + ((chunk ^ ((row >> 1) & 3)) << 4));
}

struct MmaSmem {
    size_t rings, bt, btlast, w0, bias, spins, zring, total;
};
// zring (3D networks): the spins of the last zrow * W positions, read by
// layer 0's z-plane tap
__host__ __device__ inline MmaSmem mma_layout(int D, int W, int zrow) {
    MmaSmem m{};
    const size_t slot = (size_t)kMmaRows * 64;
    m.rings = 0;
    m.bt = m.rings + (size_t)(D - 1) * (W + 2) * slot;
    m.btlast = m.bt + (size_t)(D - 2) * kC * kBtRow * 2;
    m.w0 = m.btlast + (size_t)8 * kBtRow * 2;
    m.bias = m.w0 + sizeof(float) * 4 * kC;
    m.spins = m.bias + sizeof(float) * ((size_t)(D - 1) * kC + 1);
    m.zring = m.spins + (size_t)(W + 2) * kMmaRows;
    m.total = m.zring + (size_t)zrow * W * kMmaRows;
    m.total = (m.total + 15) & ~(size_t)15;
    return m;
}

// One tap (two k-steps of 16 input channels) of a 16 x 32 ring tile into the
// 8-output-channel accumulator `acc`.  Shared-memory byte addresses: `tile` =
// the tile, `aoff0/1` = this lane's ldmatrix row/chunk offsets for k-steps 0/1,
// `wrow` = this lane's row/column in the tap's block of transposed weights.
__device__ __forceinline__ void mma_tap(float* acc, uint32_t tile, uint32_t aoff0, uint32_t aoff1,
                                        uint32_t wrow) {
    // x4 over the tap's 32 k values: (n, k0-7) (n, k8-15) (n, k16-23) (n, k24-31)
    uint32_t b0, b1, b2, b3, a0, a1, a2, a3;
    ldsm_x4(b0, b1, b2, b3, wrow);
    ldsm_x4(a0, a1, a2, a3, tile + aoff0);
    mma_bf16(acc, a0, a1, a2, a3, b0, b1);
    ldsm_x4(a0, a1, a2, a3, tile + aoff1);
    mma_bf16(acc, a0, a1, a2, a3, b2, b3);
}

// mode / flip / stream exactly as k_ar_run.  A CTA of four warps owns 16
// configurations: warp w computes output channels 8w..8w+7 of every hidden
// layer (one n-tile), so all four SM sub-partitions issue tensor instructions
// while the CTA's rings (the shared-memory limit) hold one group.  At every
// position the four taps that look back at earlier positions are accumulated
// first for all layers (independent work); only the centre tap, which needs
// the layer below at this position, stays on the layer-to-layer critical path.
// Addresses are 32-bit shared-memory offsets fixed per lane; the layer-0
// weights and the epilogue biases of a thread live in registers.
template <int D>
__global__ void __launch_bounds__(128)
    k_ar_mma(const __nv_bfloat16* __restrict__ w, NetShape S, int H, int W, int mode, int flip,
             int8_t* __restrict__ spins, float* __restrict__ logq, int n_cfg, uint64_t seed,
             uint64_t step) {
    extern __shared__ __align__(16) unsigned char smem[];
    const MmaSmem L = mma_layout(D, W, S.zrow);
    unsigned char* rings = smem + L.rings;
    int8_t* zring = reinterpret_cast<int8_t*>(smem + L.zring);
    const int zw = S.zrow * W;  // positions one z-plane back (0: 2D)
    __nv_bfloat16* bt = reinterpret_cast<__nv_bfloat16*>(smem + L.bt);
    __nv_bfloat16* btl = reinterpret_cast<__nv_bfloat16*>(smem + L.btlast);
    int8_t* sring = reinterpret_cast<int8_t*>(smem + L.spins);
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    const int ring = W + 2;
    constexpr uint32_t kSlot = kMmaRows * 64;        // bytes of one ring slot
    constexpr uint32_t kWRow = kBtRow * 2;           // bytes of one weight row
    const uint32_t lstride = (uint32_t)ring * kSlot; // bytes of one layer's ring
    const int HW = H * W;
    const int cfg0 = blockIdx.x * kMmaRows;
    // stage the weights: hidden layers l = 1..D-2 as bt[l-1][n][tap*32 + ci],
    // the last layer as btl[n][..] (only n = 0 nonzero)
    for (int l = 1; l < D - 1; ++l) {
        __nv_bfloat16* b = bt + (size_t)(l - 1) * kC * kBtRow;
        for (int i = tid; i < kC * kBtRow; i += blockDim.x) {
            const int n = i / kBtRow, k = i - n * kBtRow;
            b[i] = k < 5 * kC ? w[S.woff[l] + k * kC + n] : __float2bfloat16(0.f);
        }
    }
    for (int i = tid; i < 8 * kBtRow; i += blockDim.x) {
        const int n = i / kBtRow, k = i - n * kBtRow;
        btl[i] = (n == 0 && k < 5 * kC) ? w[S.woff[D - 1] + k] : __float2bfloat16(0.f);
    }
    // layer 0: thread = 8 r + j computes channels 4j..4j+3 of configuration r
    const int r0 = tid >> 3, j0 = tid & 7;
    float w0r[5][4], b0r[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        b0r[e] = bf(w, S.boff[0] + 4 * j0 + e);
#pragma unroll
        for (int t = 0; t < 5; ++t)
            w0r[t][e] = t < S.taps[0] ? bf(w, S.woff[0] + t * kC + 4 * j0 + e) : 0.f;
    }
    const int g = lane >> 2, q4 = lane & 3;
    // epilogue biases of this lane's two columns in every hidden layer
    float bh[D > 2 ? D - 2 : 1][2];
#pragma unroll
    for (int l = 1; l < D - 1; ++l) {
        bh[l - 1][0] = bf(w, S.boff[l] + wp * 8 + 2 * q4);
        bh[l - 1][1] = bf(w, S.boff[l] + wp * 8 + 2 * q4 + 1);
    }
    const float blast = bf(w, S.boff[D - 1]);
    __syncthreads();
    const uint32_t rings_s = smem_u32(rings);
    const uint32_t aoff0 = (uint32_t)ring_off(lane & 15, lane >> 4);
    const uint32_t aoff1 = (uint32_t)ring_off(lane & 15, 2 + (lane >> 4));
    const uint32_t blane = (uint32_t)((lane & 7) * kWRow + (lane >> 3) * 16);
    const uint32_t wbase = smem_u32(bt) + (uint32_t)(8 * wp) * kWRow + blane;
    const uint32_t wlast = smem_u32(btl) + blane;
    const uint32_t eoff0 = (uint32_t)ring_off(g, wp) + 4 * q4;
    const uint32_t eoff1 = (uint32_t)ring_off(g + 8, wp) + 4 * q4;
    const uint32_t l0off = (uint32_t)ring_off(r0, j0 >> 1) + (j0 & 1) * 8;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const uint32_t c3 = counter_word3(kTagLearn, 0, step);
    // warp 0, lanes 4g: configurations g and g+8 (logit rows of the last layer)
    const int ca = cfg0 + g, cb = cfg0 + g + 8;
    float lqa = 0.f, lqb = 0.f;
    int y = 0, x = 0, slot = 0;
    for (int p = 0; p < HW; ++p) {
        const bool up = y > 0, left = x > 0, right = x + 1 < W;
        // mask-B taps (-1,-1) (-1,0) (-1,+1) (0,-1) sit at p - W - 1 .. p - 1,
        // i.e. ring slots slot + 1, + 2, + 3 and slot - 1 (mod W + 2); the
        // centre (0,0) is `slot`
        const int ts0 = slot + 1 < ring ? slot + 1 : slot + 1 - ring;
        const int ts1 = slot + 2 < ring ? slot + 2 : slot + 2 - ring;
        const int ts2 = slot + 3 < ring ? slot + 3 : slot + 3 - ring;
        const int ts3 = slot > 0 ? slot - 1 : ring - 1;
        const bool ok0 = up && left, ok1 = up, ok2 = up && right, ok3 = left;
        const uint32_t o0 = rings_s + (uint32_t)ts0 * kSlot, o1 = rings_s + (uint32_t)ts1 * kSlot;
        const uint32_t o2 = rings_s + (uint32_t)ts2 * kSlot, o3 = rings_s + (uint32_t)ts3 * kSlot;
        const uint32_t oc = rings_s + (uint32_t)slot * kSlot;
        // phase 1: look-back taps of every layer (the last layer on warp 0)
        float acc[D - 1][4];
#pragma unroll
        for (int l = 1; l < D; ++l) {
            const bool last = l == D - 1;
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[l - 1][e] = 0.f;
            if (last && wp != 0) continue;
            const uint32_t lo = (uint32_t)(l - 1) * lstride;
            const uint32_t wr = last ? wlast : wbase + (uint32_t)((l - 1) * kC) * kWRow;
            if (ok0) mma_tap(acc[l - 1], o0 + lo, aoff0, aoff1, wr + 0 * kC * 2);
            if (ok1) mma_tap(acc[l - 1], o1 + lo, aoff0, aoff1, wr + 1 * kC * 2);
            if (ok2) mma_tap(acc[l - 1], o2 + lo, aoff0, aoff1, wr + 2 * kC * 2);
            if (ok3) mma_tap(acc[l - 1], o3 + lo, aoff0, aoff1, wr + 3 * kC * 2);
        }
        // the spin sampled at p - 1 (warp 0, end of the previous position) is
        // read by layer 0 below: the other warps did their look-back taps first
        __syncthreads();
        // layer 0 (mask A, 1 -> 32)
        {
            const float sv0 = ok0 ? (float)sring[ts0 * kMmaRows + r0] : 0.f;
            const float sv1 = ok1 ? (float)sring[ts1 * kMmaRows + r0] : 0.f;
            const float sv2 = ok2 ? (float)sring[ts2 * kMmaRows + r0] : 0.f;
            const float sv3 = ok3 ? (float)sring[ts3 * kMmaRows + r0] : 0.f;
            // z-plane tap: position p - zw, whose spin zring slot p mod zw
            // still holds (this position's spin replaces it below)
            const float sv4 = (zw > 0 && p >= zw) ? (float)zring[(p % zw) * kMmaRows + r0] : 0.f;
            float v[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float a = b0r[e];
                a = fmaf(w0r[0][e], sv0, a);
                a = fmaf(w0r[1][e], sv1, a);
                a = fmaf(w0r[2][e], sv2, a);
                a = fmaf(w0r[3][e], sv3, a);
                if (zw > 0) a = fmaf(w0r[4][e], sv4, a);
                v[e] = fmaxf(a, 0.f);
            }
            __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
            __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
            *reinterpret_cast<uint2*>(rings + (size_t)slot * kSlot + l0off) =
                make_uint2(*reinterpret_cast<uint32_t*>(&p0), *reinterpret_cast<uint32_t*>(&p1));
        }
        __syncthreads();
        // phase 2: centre tap layer by layer
#pragma unroll
        for (int l = 1; l < D; ++l) {
            const bool last = l == D - 1;
            const uint32_t in = oc + (uint32_t)(l - 1) * lstride;
            if (!last) {
                mma_tap(acc[l - 1], in, aoff0, aoff1,
                        wbase + (uint32_t)((l - 1) * kC) * kWRow + 4 * kC * 2);
                unsigned char* out = rings + (size_t)l * lstride + (size_t)slot * kSlot;
                __nv_bfloat162 lo = __floats2bfloat162_rn(fmaxf(acc[l - 1][0] + bh[l - 1][0], 0.f),
                                                          fmaxf(acc[l - 1][1] + bh[l - 1][1], 0.f));
                __nv_bfloat162 hi = __floats2bfloat162_rn(fmaxf(acc[l - 1][2] + bh[l - 1][0], 0.f),
                                                          fmaxf(acc[l - 1][3] + bh[l - 1][1], 0.f));
                *reinterpret_cast<__nv_bfloat162*>(out + eoff0) = lo;
                *reinterpret_cast<__nv_bfloat162*>(out + eoff1) = hi;
                __syncthreads();
            } else if (wp == 0) {
                mma_tap(acc[l - 1], in, aoff0, aoff1, wlast + 4 * kC * 2);
                if (q4 == 0) {
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int c = e == 0 ? ca : cb;
                        const float z = (e == 0 ? acc[l - 1][0] : acc[l - 1][2]) + blast;
                        const int row = e == 0 ? g : g + 8;
                        int8_t sv = 1;
                        if (c < n_cfg) {
                            if (mode == 0) {
                                const U4 u = philox10((uint32_t)c, (uint32_t)p, (uint32_t)step, c3,
                                                      k0, k1);
                                const float pr = 1.0f / (1.0f + __expf(-z));
                                sv = uniform24(u.x) < pr ? (int8_t)1 : (int8_t)-1;
                                spins[(size_t)c * HW + p] = sv;
                            } else {
                                sv = spins[(size_t)c * HW + p];
                                if (flip) sv = (int8_t)-sv;
                            }
                            if (e == 0)
                                lqa += log_sigmoid((float)sv * z);
                            else
                                lqb += log_sigmoid((float)sv * z);
                        }
                        sring[slot * kMmaRows + row] = sv;
                        if (zw > 0) zring[(p % zw) * kMmaRows + row] = sv;
                    }
                }
            }
        }
        // no barrier here: the next position's look-back taps read only hidden
        // layers written before the last hidden-layer barrier, and write nothing
        if (++x == W) {
            x = 0;
            ++y;
        }
        if (++slot == ring) slot = 0;
    }
    if (wp == 0 && q4 == 0) {
        if (ca < n_cfg) logq[ca] = lqa;
        if (cb < n_cfg) logq[cb] = lqb;
    }
}

// ------------------------------------- tensor-core scoring (implicit GEMM)
// log q of given configurations with every position of a layer at once: a CTA
// stages the weights once and scores configurations blockIdx.x, + gridDim.x,
// ...; rows of the tensor-core tiles = 16 positions.  Each
// output element follows exactly the sampler's chain (taps 0..4 in order,
// two k-steps each, bias after, ReLU, BF16), a tap outside the lattice adding
// an exact zero (its A row points at a zero row), and the per-position log
// sigmoid terms are summed in position order by one thread; so log q is
// bit-identical to k_ar_mma's for the same configuration.
struct ScoreSmem {
    size_t act, zero, bt, btlast, w0, bias, spin, term, total;
};
__host__ __device__ inline ScoreSmem score_layout(int D, int HW) {
    ScoreSmem m{};
    const size_t tiles = (size_t)(HW + 15) / 16;  // 16 positions x 64 B per tile
    m.act = 0;
    m.zero = m.act + 2 * tiles * 1024;
    m.bt = m.zero + 64;
    m.btlast = m.bt + (size_t)(D - 2) * kC * kBtRow * 2;
    m.w0 = m.btlast + (size_t)8 * kBtRow * 2;
    m.bias = m.w0 + sizeof(float) * 5 * kC;
    m.term = m.bias + sizeof(float) * ((size_t)(D - 1) * kC + 4);
    m.spin = m.term + sizeof(float) * (size_t)HW;
    m.total = (m.spin + (size_t)HW + 15) & ~(size_t)15;
    return m;
}

template <int D>
__global__ void __launch_bounds__(256, 1)
    k_ar_score(const __nv_bfloat16* __restrict__ w, NetShape S, int H, int W, int flip,
               const int8_t* __restrict__ spins, float* __restrict__ logq, int n_cfg) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int HW = H * W;
    const ScoreSmem L = score_layout(D, HW);
    unsigned char* act = smem + L.act;
    __nv_bfloat16* bt = reinterpret_cast<__nv_bfloat16*>(smem + L.bt);
    __nv_bfloat16* btl = reinterpret_cast<__nv_bfloat16*>(smem + L.btlast);
    float* w0 = reinterpret_cast<float*>(smem + L.w0);
    float* bias = reinterpret_cast<float*>(smem + L.bias);
    float* term = reinterpret_cast<float*>(smem + L.term);
    int8_t* sp = reinterpret_cast<int8_t*>(smem + L.spin);
    const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
    constexpr uint32_t kWRow = kBtRow * 2;
    for (int l = 1; l < D - 1; ++l) {
        __nv_bfloat16* b = bt + (size_t)(l - 1) * kC * kBtRow;
        for (int i = tid; i < kC * kBtRow; i += blockDim.x) {
            const int n = i / kBtRow, k = i - n * kBtRow;
            b[i] = k < 5 * kC ? w[S.woff[l] + k * kC + n] : __float2bfloat16(0.f);
        }
    }
    for (int i = tid; i < 8 * kBtRow; i += blockDim.x) {
        const int n = i / kBtRow, k = i - n * kBtRow;
        btl[i] = (n == 0 && k < 5 * kC) ? w[S.woff[D - 1] + k] : __float2bfloat16(0.f);
    }
    for (int i = tid; i < S.taps[0] * kC; i += blockDim.x) w0[i] = bf(w, S.woff[0] + i);
    for (int l = 0; l < D - 1; ++l)
        for (int i = tid; i < kC; i += blockDim.x) bias[l * kC + i] = bf(w, S.boff[l] + i);
    if (tid == 0) bias[(D - 1) * kC] = bf(w, S.boff[D - 1]);
    if (tid < 16) reinterpret_cast<uint32_t*>(smem + L.zero)[tid] = 0u;
    // the staged weights serve every configuration this CTA scores
    for (int c = blockIdx.x; c < n_cfg; c += gridDim.x) {
    __syncthreads();
    for (int p = tid; p < HW; p += blockDim.x) {
        const int8_t v = spins[(size_t)c * HW + p];
        sp[p] = flip ? (int8_t)-v : v;
    }
    __syncthreads();
    // layer 0 (mask A, 1 -> 32), as the sampler: a = bias; fma over taps 0..3
    // and, for a 3D network, the z-plane tap
    const int zw = S.zrow * W;
    for (int i = tid; i < HW * 4; i += blockDim.x) {
        const int p = i >> 2, j2 = i & 3;  // channels 8 j2 .. 8 j2 + 7 (one chunk)
        const int y = p / W, x = p - y * W;
        const bool up = y > 0, left = x > 0, right = x + 1 < W;
        const float s0 = (up && left) ? (float)sp[p - W - 1] : 0.f;
        const float s1 = up ? (float)sp[p - W] : 0.f;
        const float s2 = (up && right) ? (float)sp[p - W + 1] : 0.f;
        const float s3 = left ? (float)sp[p - 1] : 0.f;
        const float s4 = (zw > 0 && p >= zw) ? (float)sp[p - zw] : 0.f;
        uint32_t packed[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            float v[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int co = 8 * j2 + 2 * h + e;
                float a = bias[co];
                a = fmaf(w0[0 * kC + co], s0, a);
                a = fmaf(w0[1 * kC + co], s1, a);
                a = fmaf(w0[2 * kC + co], s2, a);
                a = fmaf(w0[3 * kC + co], s3, a);
                if (zw > 0) a = fmaf(w0[4 * kC + co], s4, a);
                v[e] = fmaxf(a, 0.f);
            }
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v[0], v[1]);
            packed[h] = *reinterpret_cast<uint32_t*>(&b2);
        }
        *reinterpret_cast<uint4*>(act + ring_off(p & 15, j2) + (size_t)(p >> 4) * 1024) =
            make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
    __syncthreads();
    const uint32_t act_s = smem_u32(act), zero_s = smem_u32(smem + L.zero);
    const int mtiles = (HW + 15) / 16;
    const uint32_t layer_bytes = (uint32_t)mtiles * 1024;
    const int g = lane >> 2, q4 = lane & 3;
    for (int l = 1; l < D; ++l) {
        const bool last = l == D - 1;
        const uint32_t in_s = act_s + (uint32_t)((l - 1) & 1) * layer_bytes;
        unsigned char* out = act + (size_t)(l & 1) * layer_bytes;
        const uint32_t wl = smem_u32(last ? btl : bt + (size_t)(l - 1) * kC * kBtRow);
        for (int mt = wp; mt < mtiles; mt += (int)(blockDim.x >> 5)) {
            // this lane's A row: position pr = 16 mt + (lane & 15)
            // (rows past the lattice read zeros; their outputs are never used)
            const int pr = mt * 16 + (lane & 15);
            const bool live = pr < HW;
            const int yr = pr / W, xr = pr - yr * W;
            const bool up = yr > 0, left = xr > 0, right = xr + 1 < W;
            const int ch = lane >> 4;  // chunk within a k-step
            uint32_t arow[5];
            const int tp[5] = {pr - W - 1, pr - W, pr - W + 1, pr - 1, pr};
            const bool tv[5] = {live && up && left, live && up, live && up && right,
                                live && left, live};
#pragma unroll
            for (int t = 0; t < 5; ++t)
                arow[t] = tv[t] ? in_s + (uint32_t)(tp[t] >> 4) * 1024 +
                                      (uint32_t)((tp[t] & 15) * 64)
                                : 0xFFFFFFFFu;
            float acc[4][4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                // B of this tap: x4 over its 32 k values for every output tile
                uint32_t bw[4][4];
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    if (last && nt > 0) break;
                    ldsm_x4(bw[nt][0], bw[nt][1], bw[nt][2], bw[nt][3],
                            wl + (uint32_t)(nt * 8 + (lane & 7)) * kWRow + (uint32_t)(t * kC) * 2 +
                                (lane >> 3) * 16);
                }
#pragma unroll
                for (int kb = 0; kb < 2; ++kb) {
                    const int chunk = 2 * kb + ch;
                    const uint32_t aaddr =
                        arow[t] == 0xFFFFFFFFu
                            ? zero_s + (uint32_t)chunk * 16
                            : arow[t] + (uint32_t)((chunk ^ ((tp[t] >> 1) & 3)) << 4);
                    uint32_t a0, a1, a2, a3;
                    ldsm_x4(a0, a1, a2, a3, aaddr);
#pragma unroll
                    for (int nt = 0; nt < 4; ++nt) {
                        if (last && nt > 0) break;
                        mma_bf16(acc[nt], a0, a1, a2, a3, bw[nt][2 * kb], bw[nt][2 * kb + 1]);
                    }
                }
            }
            if (!last) {
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int col = nt * 8 + 2 * q4;
                    const float b0 = bias[l * kC + col], b1 = bias[l * kC + col + 1];
                    __nv_bfloat162 lo = __floats2bfloat162_rn(fmaxf(acc[nt][0] + b0, 0.f),
                                                              fmaxf(acc[nt][1] + b1, 0.f));
                    __nv_bfloat162 hi = __floats2bfloat162_rn(fmaxf(acc[nt][2] + b0, 0.f),
                                                              fmaxf(acc[nt][3] + b1, 0.f));
                    unsigned char* tile = out + (size_t)mt * 1024;
                    *reinterpret_cast<__nv_bfloat162*>(tile + ring_off(g, nt) + q4 * 4) = lo;
                    *reinterpret_cast<__nv_bfloat162*>(tile + ring_off(g + 8, nt) + q4 * 4) = hi;
                }
            } else if (q4 == 0) {
                const float bl = bias[(D - 1) * kC];
                const int pa = mt * 16 + g, pb = pa + 8;
                if (pa < HW) term[pa] = log_sigmoid((float)sp[pa] * (acc[0][0] + bl));
                if (pb < HW) term[pb] = log_sigmoid((float)sp[pb] * (acc[0][2] + bl));
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        float lq = 0.f;
        for (int p = 0; p < HW; ++p) lq += term[p];
        logq[c] = lq;
    }
    }
}

__global__ void k_to_float(const int8_t* __restrict__ s, float* __restrict__ f, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        f[i] = (float)s[i];
}

}  // namespace
}  // namespace isg

using namespace isg;

struct isg_learned {
    int device = 0;
    int H = 0, W = 0, D = 6;
    uint64_t seed = 0;
    NetShape S{};
    cudaStream_t stream = nullptr;
    __nv_bfloat16* d_wbf = nullptr;
    float* d_master = nullptr;
    float* d_m1 = nullptr;
    float* d_m2 = nullptr;
    float* d_grad = nullptr;
    int64_t adam_t = 0;
    // training buffers (capacity B)
    int cap_B = 0;
    bool tc_attr = false;     // shared-memory limits of the tensor-core training kernels set
    float* d_act = nullptr;   // [D+1][B][HW][kC]: a_0 = input spins, a_l = layer l-1 output
    float* d_z = nullptr;     // [D][B][HW][kC] pre-activations
    float* d_dz = nullptr;    // [B][HW][kC]
    float* d_dz2 = nullptr;
    float* d_part = nullptr;
    float* d_lq = nullptr;
    int8_t* d_cfg = nullptr;  // [B][HW] training configurations
    int part_cap = 0;
};

namespace isg {

static int grid_for(int64_t n, int thr) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + thr - 1) / thr, 152 * 32));
}

// The tensor-core kernel when its rings and weights fit in shared memory.
static bool use_mma(const isg_learned* h) {
    return h->D >= 2 && h->D <= 8 && mma_layout(h->D, h->W, h->S.zrow).total <= 232448;
}

template <int D>
static int launch_mma(isg_learned* h, int mode, int flip, int8_t* spins, float* lq, int K,
                      uint64_t step) {
    const size_t smem = mma_layout(D, h->W, h->S.zrow).total;
    ISG_CK(cudaFuncSetAttribute(k_ar_mma<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    k_ar_mma<D><<<(K + kMmaRows - 1) / kMmaRows, 128, smem, h->stream>>>(
        h->d_wbf, h->S, h->H, h->W, mode, flip, spins, lq, K, h->seed, step);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

// Scoring with all positions of a layer at once when its buffers fit.
static bool use_score(const isg_learned* h) {
    return use_mma(h) && score_layout(h->D, h->H * h->W).total <= 232448;
}

template <int D>
static int launch_score(isg_learned* h, int flip, const int8_t* spins, float* lq, int K) {
    const size_t smem = score_layout(D, h->H * h->W).total;
    ISG_CK(cudaFuncSetAttribute(k_ar_score<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    k_ar_score<D><<<std::min(K, sms), 256, smem, h->stream>>>(h->d_wbf, h->S, h->H, h->W, flip,
                                                             spins, lq, K);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

static int launch_ar(isg_learned* h, int mode, int flip, int8_t* spins, float* lq, int K,
                     uint64_t step) {
    if (mode == 1 && use_score(h)) {
        switch (h->D) {
            case 2: return launch_score<2>(h, flip, spins, lq, K);
            case 3: return launch_score<3>(h, flip, spins, lq, K);
            case 4: return launch_score<4>(h, flip, spins, lq, K);
            case 5: return launch_score<5>(h, flip, spins, lq, K);
            case 6: return launch_score<6>(h, flip, spins, lq, K);
            case 7: return launch_score<7>(h, flip, spins, lq, K);
            default: return launch_score<8>(h, flip, spins, lq, K);
        }
    }
    if (use_mma(h)) {
        switch (h->D) {
            case 2: return launch_mma<2>(h, mode, flip, spins, lq, K, step);
            case 3: return launch_mma<3>(h, mode, flip, spins, lq, K, step);
            case 4: return launch_mma<4>(h, mode, flip, spins, lq, K, step);
            case 5: return launch_mma<5>(h, mode, flip, spins, lq, K, step);
            case 6: return launch_mma<6>(h, mode, flip, spins, lq, K, step);
            case 7: return launch_mma<7>(h, mode, flip, spins, lq, K, step);
            default: return launch_mma<8>(h, mode, flip, spins, lq, K, step);
        }
    } else {
        constexpr int G = 4;
        const size_t smem = (size_t)(h->D - 1) * (h->W + 2) * G * kC * sizeof(float) +
                            (size_t)G * h->H * h->W;
        ISG_CK(cudaFuncSetAttribute(k_ar_run<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
        k_ar_run<G><<<(K + G - 1) / G, G * kC, smem, h->stream>>>(
            h->d_wbf, h->S, h->H, h->W, mode, flip, spins, lq, K, h->seed, step);
    }
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

static int ensure_train(isg_learned* h, int B) {
    if (B <= h->cap_B) return ISG_OK;
    cudaFree(h->d_act);
    cudaFree(h->d_z);
    cudaFree(h->d_dz);
    cudaFree(h->d_dz2);
    cudaFree(h->d_lq);
    cudaFree(h->d_cfg);
    const size_t HW = (size_t)h->H * h->W;
    ISG_CK(cudaMalloc((void**)&h->d_act, sizeof(float) * (h->D + 1) * B * HW * kC));
    ISG_CK(cudaMalloc((void**)&h->d_z, sizeof(float) * h->D * B * HW * kC));
    ISG_CK(cudaMalloc((void**)&h->d_dz, sizeof(float) * B * HW * kC));
    ISG_CK(cudaMalloc((void**)&h->d_dz2, sizeof(float) * B * HW * kC));
    ISG_CK(cudaMalloc((void**)&h->d_lq, sizeof(float) * B));
    ISG_CK(cudaMalloc((void**)&h->d_cfg, (size_t)B * HW));
    h->cap_B = B;
    return ISG_OK;
}

// Forward + backward of a batch already in d_cfg; gradient into d_grad;
// mean log q into *mean_lq (if not NULL).
static int forward_backward(isg_learned* h, int B, float* mean_lq) {
    const int HW = h->H * h->W;
    const size_t stride = (size_t)B * HW * kC;
    cudaStream_t st = h->stream;
    k_to_float<<<grid_for((int64_t)B * HW, 256), 256, 0, st>>>(h->d_cfg, h->d_act, (int64_t)B * HW);
    // layers >= 1 on the tensor cores (rows of up to 256 positions fit the
    // staged tiles), layer 0 on the CUDA cores
    const bool tc = h->W <= 256;
    const int64_t M = (int64_t)B * HW;
    int sms = 1;
    ISG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    const int tc_grid = (int)std::max<int64_t>(1, std::min<int64_t>((M + kTcTile - 1) / kTcTile,
                                                                   2 * (int64_t)sms));
    const size_t fsm = tc_fwd_smem(h->W), wsm = tc_wgrad_smem(h->W);
    if (tc && !h->tc_attr) {
        ISG_CK(cudaFuncSetAttribute(k_tc_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm));
        ISG_CK(cudaFuncSetAttribute(k_tc_dgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)fsm));
        ISG_CK(cudaFuncSetAttribute(k_tc_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)wsm));
        h->tc_attr = true;
    }
    for (int l = 0; l < h->D; ++l) {
        const bool last = l == h->D - 1;
        const int64_t n = (int64_t)B * HW * h->S.cout[l];
        if (tc && l >= 1)
            k_tc_fwd<<<tc_grid, 256, fsm, st>>>(h->d_wbf, h->S, l, h->H, h->W, B,
                                                h->d_act + l * stride, h->d_z + l * stride,
                                                last ? nullptr : h->d_act + (l + 1) * stride);
        else
            k_tf_layer<<<grid_for(n, 256), 256, 0, st>>>(h->d_wbf, h->S, l, h->H, h->W, B,
                                                          h->d_act + l * stride, h->d_z + l * stride,
                                                          last ? nullptr : h->d_act + (l + 1) * stride);
    }
    // output gradient (layer D-1 pre-activation = logits)
    k_tf_out_grad<<<B, 256, 0, st>>>(h->d_z + (h->D - 1) * stride, h->d_act, HW, B, h->d_dz,
                                     h->d_lq);
    float* dz = h->d_dz;
    float* dn = h->d_dz2;
    const int chunk = 128;
    const int nparts = (int)(((int64_t)B * HW + chunk - 1) / chunk);
    size_t wg_smem = 0;
    for (int l = 0; l < h->D; ++l)
        wg_smem = std::max(wg_smem, sizeof(float) * ((size_t)chunk * h->S.cout[l] +
                                                     (size_t)(wg_halo(h->S, l, h->W) + chunk) *
                                                         h->S.cin[l]) +
                                        (size_t)chunk);
    const int nparts_tc = (int)((M + kTcChunk - 1) / kTcChunk);
    for (int l = h->D - 1; l >= 0; --l) {
        const int nw = h->S.taps[l] * h->S.cin[l] * h->S.cout[l] + h->S.cout[l];
        const bool tcl = tc && l >= 1;
        const int np = tcl ? nparts_tc : nparts;
        if ((int64_t)np * nw > h->part_cap) {
            cudaFree(h->d_part);
            h->part_cap = (int64_t)np * nw;
            ISG_CK(cudaMalloc((void**)&h->d_part, sizeof(float) * h->part_cap));
        }
        if (tcl) {
            k_tc_wgrad<<<np, 320, wsm, st>>>(h->S, l, h->H, h->W, B, h->d_act + l * stride, dz,
                                             h->d_part);
        } else {
            if (wg_smem > 48 * 1024)
                ISG_CK(cudaFuncSetAttribute(k_tf_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)wg_smem));
            k_tf_wgrad<<<np, 256, wg_smem, st>>>(h->S, l, h->H, h->W, B, h->d_act + l * stride,
                                                 dz, chunk, h->d_part);
        }
        k_sum_parts<<<(nw + 255) / 256, 256, 0, st>>>(h->d_part, np, nw,
                                                      h->d_grad + h->S.woff[l]);
        if (l > 0) {
            const int64_t n = (int64_t)B * HW * h->S.cin[l];
            if (tc && h->S.cout[l] == kC)
                k_tc_dgrad<<<tc_grid, 256, fsm, st>>>(h->d_wbf, h->S, l, h->H, h->W, B, dz,
                                                      h->d_z + (l - 1) * stride, dn);
            else
                k_tf_dgrad<<<grid_for(n, 256), 256, 0, st>>>(h->d_wbf, h->S, l, h->H, h->W, B, dz,
                                                              h->d_z + (l - 1) * stride, dn);
            std::swap(dz, dn);
        }
    }
    ISG_CK(cudaGetLastError());
    if (mean_lq) {
        std::vector<float> lq(B);
        ISG_CK(cudaMemcpyAsync(lq.data(), h->d_lq, sizeof(float) * B, cudaMemcpyDeviceToHost, st));
        ISG_CK(cudaStreamSynchronize(st));
        double s = 0;
        for (float v : lq) s += v;
        *mean_lq = (float)(s / B);
    }
    return ISG_OK;
}

}  // namespace isg

extern "C" {

int isg_learned_create(isg_learned** out, int H, int W, int layers, uint64_t seed) {
    return isg_learned_create2(out, H, W, 0, layers, seed);
}

int isg_learned_create2(isg_learned** out, int H, int W, int zrow, int layers, uint64_t seed) {
    if (!out) return fail(ISG_ERR_ARG, "isg_learned_create: out is NULL");
    *out = nullptr;
    if (H < 2 || W < 2 || H * W > 65536 || layers < 2 || layers > kMaxLayers)
        return fail(ISG_ERR_ARG, "isg_learned_create: need 2 <= H, W, H*W <= 65536, 2..8 layers");
    if (zrow < 0 || zrow >= H)
        return fail(ISG_ERR_ARG, "isg_learned_create: need 0 <= zrow < H");
    isg_learned* h = new (std::nothrow) isg_learned();
    if (!h) return fail(ISG_ERR_ARG, "isg_learned_create: out of host memory");
    cudaGetDevice(&h->device);
    h->H = H;
    h->W = W;
    h->D = layers;
    h->seed = seed;
    h->S = make_shape(layers, zrow);
    const int n = h->S.total;
    // He-style initial weights from a host generator seeded by `seed`
    std::vector<float> w(n, 0.f);
    uint64_t st = seed ^ 0x5851F42D4C957F2Dull;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < layers; ++l) {
        const int fan = h->S.taps[l] * h->S.cin[l];
        const double sc = std::sqrt(2.0 / fan) * (l == layers - 1 ? 0.1 : 1.0);
        for (int i = 0; i < h->S.taps[l] * h->S.cin[l] * h->S.cout[l]; ++i)
            w[h->S.woff[l] + i] = (float)((2.0 * next() - 1.0) * sc * std::sqrt(3.0));
    }
    std::vector<__nv_bfloat16> wb(n);
    for (int i = 0; i < n; ++i) wb[i] = __float2bfloat16(w[i]);
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_wbf, sizeof(__nv_bfloat16) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_master, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_m1, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_m2, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_grad, sizeof(float) * n);
    for (int i = 0; i < n && e == cudaSuccess; ++i) w[i] = __bfloat162float(wb[i]);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_wbf, wb.data(), sizeof(__nv_bfloat16) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_master, w.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->d_m1, 0, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMemset(h->d_m2, 0, sizeof(float) * n);
    if (e != cudaSuccess) {
        isg_learned_destroy(h);
        return cuda_fail(e, "isg_learned_create");
    }
    *out = h;
    return ISG_OK;
}

int isg_learned_destroy(isg_learned* h) {
    if (!h) return ISG_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->d_wbf);
    cudaFree(h->d_master);
    cudaFree(h->d_m1);
    cudaFree(h->d_m2);
    cudaFree(h->d_grad);
    cudaFree(h->d_act);
    cudaFree(h->d_z);
    cudaFree(h->d_dz);
    cudaFree(h->d_dz2);
    cudaFree(h->d_part);
    cudaFree(h->d_lq);
    cudaFree(h->d_cfg);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return ISG_OK;
}

int isg_learned_num_params(isg_learned* h, int* n) {
    if (!h || !n) return fail(ISG_ERR_ARG, "isg_learned_num_params: NULL argument");
    *n = h->S.total;
    return ISG_OK;
}

// Weights as FP32 (the values of the BF16 copy used by every kernel).
int isg_learned_get_weights(isg_learned* h, float* w) {
    if (!h || !w) return fail(ISG_ERR_ARG, "isg_learned_get_weights: NULL argument");
    cudaSetDevice(h->device);
    std::vector<__nv_bfloat16> b(h->S.total);
    ISG_CK(cudaMemcpyAsync(b.data(), h->d_wbf, sizeof(__nv_bfloat16) * b.size(),
                           cudaMemcpyDeviceToHost, h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < b.size(); ++i) w[i] = __bfloat162float(b[i]);
    return ISG_OK;
}

int isg_learned_set_weights(isg_learned* h, const float* w) {
    if (!h || !w) return fail(ISG_ERR_ARG, "isg_learned_set_weights: NULL argument");
    cudaSetDevice(h->device);
    const int n = h->S.total;
    std::vector<__nv_bfloat16> b(n);
    std::vector<float> m(n);
    for (int i = 0; i < n; ++i) {
        b[i] = __float2bfloat16(w[i]);
        m[i] = __bfloat162float(b[i]);
    }
    ISG_CK(cudaMemcpyAsync(h->d_wbf, b.data(), sizeof(__nv_bfloat16) * n, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaMemcpyAsync(h->d_master, m.data(), sizeof(float) * n, cudaMemcpyHostToDevice,
                           h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

// Gradient of the mean negative log-likelihood over B host configurations
// (natural layout, +-1 bytes) with respect to the weights; *nll = the mean.
int isg_learned_gradient(isg_learned* h, const int8_t* cfg, int B, float* grad, float* nll) {
    if (!h || !cfg || !grad || B < 1) return fail(ISG_ERR_ARG, "isg_learned_gradient: bad argument");
    cudaSetDevice(h->device);
    int rc = ensure_train(h, B);
    if (rc) return rc;
    const size_t HW = (size_t)h->H * h->W;
    ISG_CK(cudaMemcpyAsync(h->d_cfg, cfg, (size_t)B * HW, cudaMemcpyHostToDevice, h->stream));
    float mlq = 0.f;
    rc = forward_backward(h, B, &mlq);
    if (rc) return rc;
    ISG_CK(cudaMemcpyAsync(grad, h->d_grad, sizeof(float) * h->S.total, cudaMemcpyDeviceToHost,
                           h->stream));
    ISG_CK(cudaStreamSynchronize(h->stream));
    if (nll) *nll = -mlq;
    return ISG_OK;
}

// Adam steps on configurations in device memory d_cfg_all (n configurations,
// natural layout): each step takes batch B of them in order (cyclic).
// Returns the mean log-likelihood of the last batch.
int isg_learned_train(isg_learned* h, const int8_t* d_cfg_all, int n, int B, int steps, float lr,
                      float* last_mean_logq) {
    if (!h || !d_cfg_all || n < 1 || B < 1 || steps < 0 || !(lr > 0.f))
        return fail(ISG_ERR_ARG, "isg_learned_train: bad argument");
    cudaSetDevice(h->device);
    int rc = ensure_train(h, B);
    if (rc) return rc;
    const size_t HW = (size_t)h->H * h->W;
    const int nw = h->S.total;
    float mlq = 0.f;
    int64_t pos = 0;
    for (int s = 0; s < steps; ++s) {
        for (int b = 0; b < B; ++b) {
            ISG_CK(cudaMemcpyAsync(h->d_cfg + (size_t)b * HW, d_cfg_all + (size_t)(pos % n) * HW,
                                   HW, cudaMemcpyDeviceToDevice, h->stream));
            ++pos;
        }
        rc = forward_backward(h, B, s == steps - 1 ? &mlq : nullptr);
        if (rc) return rc;
        ++h->adam_t;
        const float b1 = 0.9f, b2 = 0.999f;
        const float bc1 = 1.f - std::pow(b1, (float)h->adam_t);
        const float bc2 = 1.f - std::pow(b2, (float)h->adam_t);
        k_adam<<<(nw + 255) / 256, 256, 0, h->stream>>>(h->d_master, h->d_wbf, h->d_grad, h->d_m1,
                                                       h->d_m2, nw, lr, b1, b2, 1e-8f, bc1, bc2);
    }
    ISG_CK(cudaGetLastError());
    ISG_CK(cudaStreamSynchronize(h->stream));
    if (last_mean_logq) *last_mean_logq = mlq;
    return ISG_OK;
}

// Draw K configurations from q (sampling mode) into d_out (device, natural
// layout) with their log q, and log q of the flipped configurations (scoring
// mode of the same kernel) into d_lq_flip.  step selects the Philox stream.
int isg_learned_sample(isg_learned* h, int K, uint64_t step, int8_t* d_out, float* d_lq,
                       float* d_lq_flip) {
    if (!h || !d_out || !d_lq || K < 1) return fail(ISG_ERR_ARG, "isg_learned_sample: bad argument");
    cudaSetDevice(h->device);
    int rc = launch_ar(h, 0, 0, d_out, d_lq, K, step);
    if (!rc && d_lq_flip) rc = launch_ar(h, 1, 1, d_out, d_lq_flip, K, step);
    return rc;
}

// Proposals per full wave of the sampling kernel: configurations per CTA x
// resident CTAs per SM x SMs.  A sampling pass costs the same for any K up to
// a multiple of this, so batches sized in these units waste no SM.
int isg_learned_batch_quantum(isg_learned* h, int* quantum) {
    if (!h || !quantum) return fail(ISG_ERR_ARG, "isg_learned_batch_quantum: bad argument");
    cudaSetDevice(h->device);
    int sms = 1;
    ISG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    int per_sm = 1, rows = kMmaRows;
    if (use_mma(h)) {
        const size_t smem = mma_layout(h->D, h->W, h->S.zrow).total;
        void (*k)(const __nv_bfloat16*, NetShape, int, int, int, int, int8_t*, float*, int,
                  uint64_t, uint64_t) = nullptr;
        switch (h->D) {
            case 2: k = k_ar_mma<2>; break;
            case 3: k = k_ar_mma<3>; break;
            case 4: k = k_ar_mma<4>; break;
            case 5: k = k_ar_mma<5>; break;
            case 6: k = k_ar_mma<6>; break;
            case 7: k = k_ar_mma<7>; break;
            default: k = k_ar_mma<8>; break;
        }
        ISG_CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ISG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, smem));
    } else {
        rows = 4;  // the CUDA-core kernel: 4 configurations per block
        per_sm = 1;
    }
    *quantum = rows * std::max(per_sm, 1) * sms;
    return ISG_OK;
}

// log q of K given configurations (device, natural layout): scoring mode of
// the sampling kernel; flip = 1 scores the negated configurations.
int isg_learned_score(isg_learned* h, const int8_t* d_cfg, int K, int flip, float* d_lq) {
    if (!h || !d_cfg || !d_lq || K < 1) return fail(ISG_ERR_ARG, "isg_learned_score: bad argument");
    cudaSetDevice(h->device);
    return launch_ar(h, 1, flip ? 1 : 0, const_cast<int8_t*>(d_cfg), d_lq, K, 0);
}

// Exact energies (bond sum, magnetisation) of K configurations of a periodic
// L^dim lattice in device memory.
int isg_learned_energies(isg_learned* h, const int8_t* d_cfg, int K, int L, int dim,
                         int64_t* d_bond, int64_t* d_mag) {
    if (!h || !d_cfg || !d_bond || !d_mag || K < 1 || (dim != 2 && dim != 3))
        return fail(ISG_ERR_ARG, "isg_learned_energies: bad argument");
    cudaSetDevice(h->device);
    k_cfg_energy<<<K, 256, 0, h->stream>>>(d_cfg, L, dim, K, (long long*)d_bond, (long long*)d_mag);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

// One independence Metropolis-Hastings pass over K proposals (k_imh_prep +
// k_imh_scan).  d_state = (bond, mag, index): on return index is the
// proposal the chain ends on, or -1 if it kept its state; d_ax = A of the
// current state (-beta E - log q_sym); d_mrec[k] = |M| after proposal k;
// d_brec[k] (may be NULL) = bond sum after proposal k; d_accepted accumulates
// acceptances; d_work holds 2K doubles.
int isg_learned_imh(isg_learned* h, const int64_t* d_bond, const int64_t* d_mag,
                    const float* d_lq, const float* d_lq_flip, int K, double beta, double J,
                    int64_t* d_state, double* d_ax, int64_t* d_mrec, int64_t* d_brec,
                    int64_t* d_accepted, double* d_work, uint64_t step) {
    if (!h || !d_bond || !d_mag || !d_lq || !d_lq_flip || !d_state || !d_ax || !d_mrec ||
        !d_accepted || !d_work || K < 1)
        return fail(ISG_ERR_ARG, "isg_learned_imh: bad argument");
    cudaSetDevice(h->device);
    k_imh_prep<<<(K + 127) / 128, 128, 0, h->stream>>>((const long long*)d_bond, d_lq, d_lq_flip, K,
                                                      beta, J, d_work, d_work + K, h->seed, step);
    k_imh_scan<<<1, 32, 0, h->stream>>>((const long long*)d_bond, (const long long*)d_mag, d_work,
                                        d_work + K, K, (long long*)d_state, d_ax,
                                        (long long*)d_mrec, (long long*)d_brec,
                                        (long long*)d_accepted);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

// A = -beta E - log q_sym for one configuration whose bond sum is known,
// from its log q and log q of its negation (device scalars).
__global__ void k_state_a(const float* __restrict__ lq, const float* __restrict__ lqf,
                          const long long* __restrict__ bond, double beta, double J,
                          double* __restrict__ ax) {
    const double la = lq[0], lb = lqf[0];
    const double mx = la > lb ? la : lb;
    const double lsym = mx + log(0.5 * (exp(la - mx) + exp(lb - mx)));
    *ax = -beta * (-J * (double)bond[0]) - lsym;
}

int isg_learned_state_a(isg_learned* h, const float* d_lq, const float* d_lq_flip,
                        const int64_t* d_bond, double beta, double J, double* d_ax) {
    if (!h || !d_lq || !d_lq_flip || !d_bond || !d_ax)
        return fail(ISG_ERR_ARG, "isg_learned_state_a: NULL argument");
    cudaSetDevice(h->device);
    k_state_a<<<1, 1, 0, h->stream>>>(d_lq, d_lq_flip, (const long long*)d_bond, beta, J, d_ax);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

int isg_learned_adopt(isg_learned* h, const int8_t* d_props, const int64_t* d_state,
                      int8_t* d_current) {
    if (!h || !d_props || !d_state || !d_current)
        return fail(ISG_ERR_ARG, "isg_learned_adopt: NULL argument");
    cudaSetDevice(h->device);
    const int n = h->H * h->W;
    k_adopt<<<(n + 255) / 256, 256, 0, h->stream>>>(d_props, (const long long*)d_state, d_current,
                                                    n);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

int isg_learned_sync(isg_learned* h) {
    if (!h) return fail(ISG_ERR_ARG, "isg_learned_sync: NULL handle");
    cudaSetDevice(h->device);
    ISG_CK(cudaStreamSynchronize(h->stream));
    return ISG_OK;
}

void* isg_learned_stream(isg_learned* h) { return h ? (void*)h->stream : nullptr; }

}  // extern "C"
