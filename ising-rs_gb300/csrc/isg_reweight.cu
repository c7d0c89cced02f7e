// isg_reweight.cu — Ferrenberg-Swendsen reweighting on the GPU: the
// multiple-histogram (WHAM) free-energy iteration and reweighted averages at
// target temperatures, over samples or over energy histograms.
//
// Reference path being replaced (faulknco/ising-rs):
//   analysis/scripts/reweighting.py:15-43    single_histogram, reweight_observable
//   analysis/scripts/reweighting.py:45-105   wham_reweight (f_k iteration, weights)
//   analysis/scripts/reweighting.py:108-143  reweight_binder
//   analysis/scripts/analyze_gpu_fss.py:86-277
//                                            reweight_single_histogram and
//                                            wham_reweight_fine (observables on a
//                                            fine T grid)
//
// Points p carry an energy E_p, a weight c_p (1 for a sample; the count of an
// energy bin for a histogram) and n_mom moment sums (the point's sums of |m|,
// m^2, m^4, ...).  A histogram with exact energy bins (the Ising bond sum)
// gives the same WHAM solution and averages as its samples, because every
// sample of a bin has the same weight.
//
// WHAM as the reference iterates it: with a_k = log N_k + f_k,
//   log_denom_p = logsumexp_k (a_k - beta_k E_p)
//   f_k' = -logsumexp_p (log c_p - beta_k E_p - log_denom_p),  f' -= f'_0
// until max |f' - f| < tol (at most n_iter rounds); the weights then use the
// log_denom of the last round, as the reference does.  Averages at beta_t:
//   <O> = sum_p exp(x_p - X) O_p / sum_p exp(x_p - X) c_p,
//   x_p = -beta_t E_p - log_denom_p (WHAM) or -(beta_t - beta_k) E_p over the
//   points of simulation k (single histogram), X = max_p x_p.
//
// GPU form: one thread per point for log_denom (a loop over the K
// simulations); for f', blocks over (simulation, slice of the points) whose
// running log-sum-exps merge in slice order; one block per target for the
// averages.  Every sum runs over a fixed partition in a fixed tree, so results
// do not depend on timing.  FP64 throughout (the exponents reach 10^5-10^6).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "isg_common.cuh"

namespace isg {

constexpr int kRwThreads = 256;
constexpr int kRwMaxMom = 8;

// (m, s) represents m + log s; merge two running log-sum-exps.  A side more
// than kLseCut below the other only rescales or drops (see k_rw_denom).
__device__ __forceinline__ void lse_merge(double& m, double& s, double m2, double s2) {
    if (s2 == 0.0) return;
    if (s == 0.0) {
        m = m2;
        s = s2;
        return;
    }
    if (m2 > m) {
        s = (m - m2 > -40.0 ? s * exp(m - m2) : 0.0) + s2;
        m = m2;
    } else if (m2 - m > -40.0) {
        s = s + s2 * exp(m2 - m);
    }
}

// Terms more than kLseCut below the largest of a log-sum-exp are left out:
// e^-40 = 4e-18 is below half an ulp of the sum (>= 1), so an FP64 sum changes
// by at most an ulp while most of the exp calls (on the slow FP64 pipe) go away.
constexpr double kLseCut = 40.0;

__global__ void k_rw_denom(const double* __restrict__ e, int64_t P, const double* __restrict__ a,
                           const double* __restrict__ beta, int K, double* __restrict__ ld) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P;
         p += (int64_t)gridDim.x * blockDim.x) {
        const double E = e[p];
        double mx = -INFINITY;
        for (int k = 0; k < K; ++k) mx = fmax(mx, a[k] - beta[k] * E);
        double s = 0.0;
        for (int k = 0; k < K; ++k) {
            const double d = a[k] - beta[k] * E - mx;
            if (d > -kLseCut) s += exp(d);
        }
        ld[p] = mx + log(s);
    }
}

// Block-wide merge of per-thread (m, s) pairs; result in thread 0.
__device__ __forceinline__ void block_lse(double& m, double& s, double* sm, double* ss) {
    for (int o = 16; o > 0; o >>= 1) {
        const double m2 = __shfl_down_sync(ISG_FULL_MASK, m, o);
        const double s2 = __shfl_down_sync(ISG_FULL_MASK, s, o);
        lse_merge(m, s, m2, s2);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sm[w] = m;
        ss[w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool in = threadIdx.x < (blockDim.x >> 5);
        m = in ? sm[threadIdx.x] : 0.0;
        s = in ? ss[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            const double m2 = __shfl_down_sync(ISG_FULL_MASK, m, o);
            const double s2 = __shfl_down_sync(ISG_FULL_MASK, s, o);
            lse_merge(m, s, m2, s2);
        }
    }
}

// Partial log-sum-exps of f_k' = -logsumexp_p (log c_p - beta_k E_p - ld_p):
// block (k, g) covers the g-th of gridDim.y equal slices of the points and
// writes (m, s) to part[(k * gridDim.y + g) * 2].
__global__ void k_rw_fnew_part(const double* __restrict__ e, const double* __restrict__ c,
                               int64_t P, const double* __restrict__ ld,
                               const double* __restrict__ beta, double* __restrict__ part) {
    __shared__ double sm[32], ss[32];
    const int k = blockIdx.x, g = blockIdx.y, G = gridDim.y;
    const int64_t per = (P + G - 1) / G;
    const int64_t lo = (int64_t)g * per, hi = min(P, lo + per);
    const double bk = beta[k];
    double m = 0.0, s = 0.0;
    for (int64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
        const double cp = c[p];
        if (!(cp > 0.0)) continue;
        lse_merge(m, s, (cp == 1.0 ? 0.0 : log(cp)) - bk * e[p] - ld[p], 1.0);
    }
    block_lse(m, s, sm, ss);
    if (threadIdx.x == 0) {
        part[2 * ((size_t)k * G + g)] = m;
        part[2 * ((size_t)k * G + g) + 1] = s;
    }
}

// Merge the G partials of every k in slice order: fnew[k] = -(m + log s).
__global__ void k_rw_fnew_merge(const double* __restrict__ part, int K, int G,
                                double* __restrict__ fnew) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
        double m = 0.0, s = 0.0;
        for (int g = 0; g < G; ++g)
            lse_merge(m, s, part[2 * ((size_t)k * G + g)], part[2 * ((size_t)k * G + g) + 1]);
        fnew[k] = s > 0.0 ? -(m + log(s)) : INFINITY;
    }
}

// Averages at target t (one block per target): out[t*(3+n_mom) + ...] =
// {log Z, <E>, <E^2>, <mom_0>, ...} with Z = sum_p exp(x_p) c_p and
// <mom_j> = sum_p exp(x_p) mom_pj / Z.  mode 0: WHAM (x = -beta_t E - ld);
// mode 1: single histogram over points [p0[t], p1[t]) except [x0[t], x1[t])
// (x0, x1 may be NULL) with x = -(beta_t - bref[t]) E.
__global__ void k_rw_obs(const double* __restrict__ e, const double* __restrict__ c,
                         const double* __restrict__ mom, int n_mom, int64_t P,
                         const double* __restrict__ ld, const double* __restrict__ bt,
                         const double* __restrict__ bref, const int64_t* __restrict__ p0,
                         const int64_t* __restrict__ p1, const int64_t* __restrict__ x0,
                         const int64_t* __restrict__ x1, int mode, double* __restrict__ out) {
    __shared__ double sm[32];
    __shared__ double s_max;
    __shared__ double red[kRwMaxMom + 3][32];
    const int t = blockIdx.x;
    const double b = bt[t];
    const int64_t lo = mode == 1 ? p0[t] : 0, hi = mode == 1 ? p1[t] : P;
    const double db = mode == 1 ? b - bref[t] : 0.0;
    const int64_t xlo = (mode == 1 && x0) ? x0[t] : 0, xhi = (mode == 1 && x1) ? x1[t] : 0;
    // pass 1: max exponent
    double mx = -INFINITY;
    for (int64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
        if (!(c[p] > 0.0) || (p >= xlo && p < xhi)) continue;
        const double x = mode == 1 ? -db * e[p] : -b * e[p] - ld[p];
        mx = fmax(mx, x);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(ISG_FULL_MASK, mx, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = -INFINITY;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, sm[w]);
        s_max = v;
    }
    __syncthreads();
    const double X = s_max;
    // pass 2: shifted sums
    double acc[kRwMaxMom + 3];
    for (int j = 0; j < n_mom + 3; ++j) acc[j] = 0.0;
    for (int64_t p = lo + threadIdx.x; p < hi; p += blockDim.x) {
        if (!(c[p] > 0.0) || (p >= xlo && p < xhi)) continue;
        const double x = mode == 1 ? -db * e[p] : -b * e[p] - ld[p];
        if (x - X <= -kLseCut) continue;
        const double w = exp(x - X);
        const double wc = w * c[p];
        acc[0] += wc;
        acc[1] += wc * e[p];
        acc[2] += wc * e[p] * e[p];
        for (int j = 0; j < n_mom; ++j) acc[3 + j] += w * mom[p * n_mom + j];
    }
    for (int j = 0; j < n_mom + 3; ++j) {
        double v = acc[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(ISG_FULL_MASK, v, o);
        if ((threadIdx.x & 31) == 0) red[j][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot[kRwMaxMom + 3];
        for (int j = 0; j < n_mom + 3; ++j) {
            double v = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[j][w];
            tot[j] = v;
        }
        double* o = out + (size_t)t * (n_mom + 3);
        o[0] = X + log(tot[0]);
        o[1] = tot[1] / tot[0];
        o[2] = tot[2] / tot[0];
        for (int j = 0; j < n_mom; ++j) o[3 + j] = tot[3 + j] / tot[0];
    }
}

// Normalised weights of every point at one target (the reference's w array):
// w_p = exp(x_p - log Z) c_p with log Z from k_rw_obs.
__global__ void k_rw_weights(const double* __restrict__ e, const double* __restrict__ c, int64_t P,
                             const double* __restrict__ ld, double b,
                             const double* __restrict__ logz, double* __restrict__ w) {
    const double lz = logz[0];
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < P;
         p += (int64_t)gridDim.x * blockDim.x)
        w[p] = c[p] > 0.0 ? exp(-b * e[p] - ld[p] - lz) * c[p] : 0.0;
}

struct RwBuf {
    double *e = nullptr, *c = nullptr, *mom = nullptr, *ld = nullptr, *a = nullptr,
           *beta = nullptr, *fnew = nullptr, *bt = nullptr, *bref = nullptr, *out = nullptr,
           *w = nullptr, *part = nullptr;
    int64_t *p0 = nullptr, *p1 = nullptr, *x0 = nullptr, *x1 = nullptr;
    ~RwBuf() {
        for (double* p : {e, c, mom, ld, a, beta, fnew, bt, bref, out, w, part}) cudaFree(p);
        for (int64_t* p : {p0, p1, x0, x1}) cudaFree(p);
    }
};

int rw_grid(int64_t P) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::max<int64_t>(1, std::min<int64_t>((P + kRwThreads - 1) / kRwThreads,
                                                       (int64_t)sms * 8));
}

// Device WHAM solve; leaves the last round's log_denom in B.ld.
int rw_solve(RwBuf& B, const double* beta, const double* n_k, int K, int64_t P, int n_iter,
             double tol, double* f_out, int* iters_out, cudaStream_t st) {
    std::vector<double> f(K, 0.0), fn(K), a(K);
    int it = 0;
    const int grid = rw_grid(P);
    // slices per simulation: about four blocks per SM in all, at least 2048
    // points per slice
    int sms = 1, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int G = (int)std::max<int64_t>(
        1, std::min<int64_t>((4 * (int64_t)sms + K - 1) / K, (P + 2047) / 2048));
    ISG_CK(cudaMalloc((void**)&B.part, sizeof(double) * 2 * (size_t)K * G));
    for (it = 0; it < std::max(1, n_iter); ++it) {
        for (int k = 0; k < K; ++k) a[k] = std::log(n_k[k]) + f[k];
        ISG_CK(cudaMemcpyAsync(B.a, a.data(), sizeof(double) * K, cudaMemcpyHostToDevice, st));
        k_rw_denom<<<grid, kRwThreads, 0, st>>>(B.e, P, B.a, B.beta, K, B.ld);
        ISG_CK(cudaGetLastError());
        k_rw_fnew_part<<<dim3(K, G), kRwThreads, 0, st>>>(B.e, B.c, P, B.ld, B.beta, B.part);
        ISG_CK(cudaGetLastError());
        k_rw_fnew_merge<<<(K + 127) / 128, 128, 0, st>>>(B.part, K, G, B.fnew);
        ISG_CK(cudaGetLastError());
        ISG_CK(cudaMemcpyAsync(fn.data(), B.fnew, sizeof(double) * K, cudaMemcpyDeviceToHost, st));
        ISG_CK(cudaStreamSynchronize(st));
        const double f0 = fn[0];
        double dmax = 0.0;
        for (int k = 0; k < K; ++k) {
            fn[k] -= f0;
            dmax = std::max(dmax, std::fabs(fn[k] - f[k]));
        }
        f = fn;
        if (dmax < tol) {
            ++it;
            break;
        }
    }
    if (f_out) std::copy(f.begin(), f.end(), f_out);
    if (iters_out) *iters_out = it;
    return ISG_OK;
}

int rw_upload(RwBuf& B, const double* e, const double* c, const double* mom, int n_mom, int64_t P,
              const double* beta, int K, cudaStream_t st) {
    ISG_CK(cudaMalloc((void**)&B.e, sizeof(double) * std::max<int64_t>(P, 1)));
    ISG_CK(cudaMalloc((void**)&B.c, sizeof(double) * std::max<int64_t>(P, 1)));
    ISG_CK(cudaMalloc((void**)&B.ld, sizeof(double) * std::max<int64_t>(P, 1)));
    ISG_CK(cudaMalloc((void**)&B.mom, sizeof(double) * std::max<int64_t>(P * n_mom, 1)));
    ISG_CK(cudaMalloc((void**)&B.a, sizeof(double) * std::max(K, 1)));
    ISG_CK(cudaMalloc((void**)&B.beta, sizeof(double) * std::max(K, 1)));
    ISG_CK(cudaMalloc((void**)&B.fnew, sizeof(double) * std::max(K, 1)));
    ISG_CK(cudaMemcpyAsync(B.e, e, sizeof(double) * P, cudaMemcpyHostToDevice, st));
    ISG_CK(cudaMemcpyAsync(B.c, c, sizeof(double) * P, cudaMemcpyHostToDevice, st));
    if (n_mom > 0)
        ISG_CK(cudaMemcpyAsync(B.mom, mom, sizeof(double) * P * n_mom, cudaMemcpyHostToDevice, st));
    if (K > 0)
        ISG_CK(cudaMemcpyAsync(B.beta, beta, sizeof(double) * K, cudaMemcpyHostToDevice, st));
    return ISG_OK;
}

int rw_check(const double* e, const double* c, int64_t P, int n_mom, const double* mom,
             const char* who) {
    if (P < 1 || !e || !c) return fail(ISG_ERR_ARG, std::string(who) + ": need at least one point");
    if (n_mom < 0 || n_mom > kRwMaxMom || (n_mom > 0 && !mom))
        return fail(ISG_ERR_ARG, std::string(who) + ": n_mom must be 0..8 with moment sums");
    return ISG_OK;
}

}  // namespace isg

using namespace isg;

extern "C" {

int isg_wham(const double* e, const double* c, const double* mom, int n_mom, int64_t P,
             const double* beta, const double* n_k, int K, int n_iter, double tol,
             const double* beta_t, int T, double* out, double* f_out, int* iters_out) {
    int rc = rw_check(e, c, P, n_mom, mom, "isg_wham");
    if (rc) return rc;
    if (K < 1 || !beta || !n_k) return fail(ISG_ERR_ARG, "isg_wham: need at least one simulation");
    for (int k = 0; k < K; ++k)
        if (!(n_k[k] > 0.0)) return fail(ISG_ERR_ARG, "isg_wham: every simulation needs samples");
    if (T < 0 || (T > 0 && (!beta_t || !out))) return fail(ISG_ERR_ARG, "isg_wham: bad targets");
    cudaStream_t st = nullptr;
    ISG_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    RwBuf B;
    rc = rw_upload(B, e, c, mom, n_mom, P, beta, K, st);
    if (!rc) rc = rw_solve(B, beta, n_k, K, P, n_iter, tol, f_out, iters_out, st);
    if (!rc && T > 0) {
        cudaError_t ce = cudaMalloc((void**)&B.bt, sizeof(double) * T);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.out, sizeof(double) * T * (3 + n_mom));
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.bt, beta_t, sizeof(double) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess) {
            k_rw_obs<<<T, kRwThreads, 0, st>>>(B.e, B.c, B.mom, n_mom, P, B.ld, B.bt, nullptr,
                                               nullptr, nullptr, nullptr, nullptr, 0, B.out);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(out, B.out, sizeof(double) * T * (3 + n_mom),
                                 cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "isg_wham");
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}

int isg_wham_weights(const double* e, const double* c, int64_t P, const double* beta,
                     const double* n_k, int K, int n_iter, double tol, double beta_t, double* w,
                     double* f_out, int* iters_out) {
    int rc = rw_check(e, c, P, 0, nullptr, "isg_wham_weights");
    if (rc) return rc;
    if (K < 1 || !beta || !n_k || !w)
        return fail(ISG_ERR_ARG, "isg_wham_weights: bad arguments");
    for (int k = 0; k < K; ++k)
        if (!(n_k[k] > 0.0))
            return fail(ISG_ERR_ARG, "isg_wham_weights: every simulation needs samples");
    cudaStream_t st = nullptr;
    ISG_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    RwBuf B;
    rc = rw_upload(B, e, c, nullptr, 0, P, beta, K, st);
    if (!rc) rc = rw_solve(B, beta, n_k, K, P, n_iter, tol, f_out, iters_out, st);
    if (!rc) {
        // log Z from the averages kernel (one target), then the weights
        cudaError_t ce = cudaMalloc((void**)&B.bt, sizeof(double));
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.out, sizeof(double) * 3);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.w, sizeof(double) * P);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.bt, &beta_t, sizeof(double), cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess) {
            k_rw_obs<<<1, kRwThreads, 0, st>>>(B.e, B.c, B.mom, 0, P, B.ld, B.bt, nullptr, nullptr,
                                               nullptr, nullptr, nullptr, 0, B.out);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) {
            k_rw_weights<<<rw_grid(P), kRwThreads, 0, st>>>(B.e, B.c, P, B.ld, beta_t, B.out, B.w);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(w, B.w, sizeof(double) * P, cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "isg_wham_weights");
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}

int isg_reweight_single(const double* e, const double* c, const double* mom, int n_mom, int64_t P,
                        const int64_t* p0, const int64_t* p1, const int64_t* x0, const int64_t* x1,
                        const double* beta_ref, const double* beta_t, int T, double* out) {
    int rc = rw_check(e, c, P, n_mom, mom, "isg_reweight_single");
    if (rc) return rc;
    if (T < 1 || !p0 || !p1 || !beta_ref || !beta_t || !out || (!x0) != (!x1))
        return fail(ISG_ERR_ARG, "isg_reweight_single: bad targets");
    for (int t = 0; t < T; ++t) {
        if (p0[t] < 0 || p1[t] > P || p0[t] >= p1[t])
            return fail(ISG_ERR_ARG, "isg_reweight_single: empty or bad point range");
        if (x0 && (x0[t] > x1[t] || (x0[t] <= p0[t] && x1[t] >= p1[t])))
            return fail(ISG_ERR_ARG, "isg_reweight_single: the excluded range leaves no point");
    }
    cudaStream_t st = nullptr;
    ISG_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    RwBuf B;
    rc = rw_upload(B, e, c, mom, n_mom, P, nullptr, 0, st);
    if (!rc) {
        cudaError_t ce = cudaMalloc((void**)&B.bt, sizeof(double) * T);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.bref, sizeof(double) * T);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.p0, sizeof(int64_t) * T);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.p1, sizeof(int64_t) * T);
        if (ce == cudaSuccess && x0) ce = cudaMalloc((void**)&B.x0, sizeof(int64_t) * T);
        if (ce == cudaSuccess && x0) ce = cudaMalloc((void**)&B.x1, sizeof(int64_t) * T);
        if (ce == cudaSuccess) ce = cudaMalloc((void**)&B.out, sizeof(double) * T * (3 + n_mom));
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.bt, beta_t, sizeof(double) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.bref, beta_ref, sizeof(double) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.p0, p0, sizeof(int64_t) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(B.p1, p1, sizeof(int64_t) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess && x0)
            ce = cudaMemcpyAsync(B.x0, x0, sizeof(int64_t) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess && x0)
            ce = cudaMemcpyAsync(B.x1, x1, sizeof(int64_t) * T, cudaMemcpyHostToDevice, st);
        if (ce == cudaSuccess) {
            k_rw_obs<<<T, kRwThreads, 0, st>>>(B.e, B.c, B.mom, n_mom, P, nullptr, B.bt, B.bref,
                                               B.p0, B.p1, B.x0, B.x1, 1, B.out);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(out, B.out, sizeof(double) * T * (3 + n_mom),
                                 cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "isg_reweight_single");
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    return rc;
}

}  // extern "C"
