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
constexpr int kTaps = 5;       // (-1,-1) (-1,0) (-1,+1) (0,-1) (0,0)
__host__ __device__ __forceinline__ int tap_dy(int t) { return t < 3 ? -1 : 0; }
__host__ __device__ __forceinline__ int tap_dx(int t) { return t < 3 ? t - 1 : (t == 3 ? -1 : 0); }
constexpr uint32_t kTagLearn = 0x06u;

// Weight layout per layer l: w[tap][cin][cout] (taps 0..3 for layer 0, else
// 0..4), then bias[cout].  cin = 1 for layer 0, cout = 1 for the last layer.
struct NetShape {
    int D;                       // layers
    int cin[kMaxLayers], cout[kMaxLayers], taps[kMaxLayers];
    int woff[kMaxLayers];        // offset of layer weights
    int boff[kMaxLayers];        // offset of layer bias
    int total;
};

NetShape make_shape(int D) {
    NetShape s{};
    s.D = D;
    int off = 0;
    for (int l = 0; l < D; ++l) {
        s.cin[l] = l == 0 ? 1 : kC;
        s.cout[l] = l == D - 1 ? 1 : kC;
        s.taps[l] = l == 0 ? 4 : 5;
        s.woff[l] = off;
        off += s.taps[l] * s.cin[l] * s.cout[l];
        s.boff[l] = off;
        off += s.cout[l];
    }
    s.total = off;
    return s;
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
                    const int yy = y + tap_dy(t), xx = x + tap_dx(t);
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
            const int yy = y + tap_dy(t), xx = x + tap_dx(t);
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
            const int yy = y - tap_dy(t), xx = x - tap_dx(t);
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
__global__ void k_tf_wgrad(NetShape S, int l, int H, int W, int B, const float* __restrict__ in,
                           const float* __restrict__ dz, int chunk, float* __restrict__ part) {
    const int HW = H * W;
    const int cin = S.cin[l], cout = S.cout[l], taps = S.taps[l];
    const int nw = taps * cin * cout + cout;
    const int64_t n = (int64_t)B * HW;
    const int64_t start = (int64_t)blockIdx.x * chunk;
    const int64_t stop = start + chunk < n ? start + chunk : n;
    for (int j = threadIdx.x; j < nw; j += blockDim.x) {
        float acc = 0.f;
        if (j < taps * cin * cout) {
            const int co = j % cout;
            const int ci = (j / cout) % cin;
            const int t = j / (cout * cin);
            for (int64_t bp = start; bp < stop; ++bp) {
                const int p = (int)(bp % HW);
                const int y = p / W, x = p - y * W;
                const int yy = y + tap_dy(t), xx = x + tap_dx(t);
                if (yy < 0 || xx < 0 || xx >= W) continue;
                acc = fmaf(in[(bp - p + yy * W + xx) * cin + ci], dz[bp * cout + co], acc);
            }
        } else {
            const int co = j - taps * cin * cout;
            for (int64_t bp = start; bp < stop; ++bp) acc += dz[bp * cout + co];
        }
        part[(int64_t)blockIdx.x * nw + j] = acc;
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

static size_t ar_smem(const isg_learned* h, int G) {
    return (size_t)(h->D - 1) * (h->W + 2) * G * kC * sizeof(float) + (size_t)G * h->H * h->W;
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
    for (int l = 0; l < h->D; ++l) {
        const bool last = l == h->D - 1;
        const int64_t n = (int64_t)B * HW * h->S.cout[l];
        k_tf_layer<<<grid_for(n, 256), 256, 0, st>>>(h->d_wbf, h->S, l, h->H, h->W, B,
                                                      h->d_act + l * stride, h->d_z + l * stride,
                                                      last ? nullptr : h->d_act + (l + 1) * stride);
    }
    // output gradient (layer D-1 pre-activation = logits)
    k_tf_out_grad<<<B, 256, 0, st>>>(h->d_z + (h->D - 1) * stride, h->d_act, HW, B, h->d_dz,
                                     h->d_lq);
    float* dz = h->d_dz;
    float* dn = h->d_dz2;
    const int chunk = 2048;
    const int nparts = (int)(((int64_t)B * HW + chunk - 1) / chunk);
    for (int l = h->D - 1; l >= 0; --l) {
        const int nw = h->S.taps[l] * h->S.cin[l] * h->S.cout[l] + h->S.cout[l];
        if ((int64_t)nparts * nw > h->part_cap) {
            cudaFree(h->d_part);
            h->part_cap = nparts * nw;
            ISG_CK(cudaMalloc((void**)&h->d_part, sizeof(float) * h->part_cap));
        }
        k_tf_wgrad<<<nparts, 256, 0, st>>>(h->S, l, h->H, h->W, B, h->d_act + l * stride, dz,
                                           chunk, h->d_part);
        k_sum_parts<<<(nw + 255) / 256, 256, 0, st>>>(h->d_part, nparts, nw,
                                                      h->d_grad + h->S.woff[l]);
        if (l > 0) {
            const int64_t n = (int64_t)B * HW * h->S.cin[l];
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
    if (!out) return fail(ISG_ERR_ARG, "isg_learned_create: out is NULL");
    *out = nullptr;
    if (H < 2 || W < 2 || H * W > 65536 || layers < 2 || layers > kMaxLayers)
        return fail(ISG_ERR_ARG, "isg_learned_create: need 2 <= H, W, H*W <= 65536, 2..8 layers");
    isg_learned* h = new (std::nothrow) isg_learned();
    if (!h) return fail(ISG_ERR_ARG, "isg_learned_create: out of host memory");
    cudaGetDevice(&h->device);
    h->H = H;
    h->W = W;
    h->D = layers;
    h->seed = seed;
    h->S = make_shape(layers);
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
    constexpr int G = 4;
    const size_t smem = ar_smem(h, G);
    ISG_CK(cudaFuncSetAttribute(k_ar_run<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    const int blocks = (K + G - 1) / G;
    k_ar_run<G><<<blocks, G * kC, smem, h->stream>>>(h->d_wbf, h->S, h->H, h->W, 0, 0, d_out,
                                                      d_lq, K, h->seed, step);
    if (d_lq_flip)
        k_ar_run<G><<<blocks, G * kC, smem, h->stream>>>(h->d_wbf, h->S, h->H, h->W, 1, 1, d_out,
                                                          d_lq_flip, K, h->seed, step);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
}

// log q of K given configurations (device, natural layout): scoring mode of
// the sampling kernel; flip = 1 scores the negated configurations.
int isg_learned_score(isg_learned* h, const int8_t* d_cfg, int K, int flip, float* d_lq) {
    if (!h || !d_cfg || !d_lq || K < 1) return fail(ISG_ERR_ARG, "isg_learned_score: bad argument");
    cudaSetDevice(h->device);
    constexpr int G = 4;
    const size_t smem = ar_smem(h, G);
    ISG_CK(cudaFuncSetAttribute(k_ar_run<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    k_ar_run<G><<<(K + G - 1) / G, G * kC, smem, h->stream>>>(
        h->d_wbf, h->S, h->H, h->W, 1, flip ? 1 : 0, const_cast<int8_t*>(d_cfg), d_lq, K, h->seed,
        0);
    ISG_CK(cudaGetLastError());
    return ISG_OK;
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
