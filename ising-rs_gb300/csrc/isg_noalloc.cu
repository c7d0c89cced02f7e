// isg_noalloc.cu — observables of continuous-spin lattices without any
// allocation by the library.
//
// Some callers cannot call cudaMalloc: a host that owns every device buffer
// through its own pool allocator, code running where allocation is forbidden
// or would break an ongoing allocation budget, or a plugin that is handed
// device pointers by a framework and must not allocate behind its back.
// isg_cont_observables_static serves them: the caller passes the lattices and
// the output buffer (both device memory it owns), and the block partials that
// the reduction needs live in a fixed file-scope __device__ array instead of
// memory the library would allocate.  It computes the observables of the
// measure step of the O(n) path, summed in compensated FP32 per block with an
// FP64 combine in a fixed order (deterministic; it agrees with the exact
// fixed-point sums of isg_cont_measure to FP32 rounding), on lattices in the
// natural interleaved layout the reference uses for continuous spins (n_comp
// floats per site, site index z*L*L + y*L + x).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "isg_common.cuh"

namespace isg {
namespace {

constexpr int kObsThreads = 256;
constexpr int kObsChunk = 1024;  // sites per block
constexpr int kObsQ = 10;        // E, Mx, My, Mz, C_x, C_y, C_z, S_x, S_y, S_z
constexpr int kMaxDevices = 64;

// Scratch for the block partials: kObsMaxChunks chunks of kObsChunk sites,
// i.e. at most 16,777,216 sites per call (e.g. 8 lattices of 128^3), 1.25 MiB
// on every GPU that loads this library, held until the process exits.
constexpr int kObsMaxChunks = 16384;
static __device__ __align__(256) double g_obs_partials[kObsMaxChunks * kObsQ];

struct CFs {
    float s, c;
};
__device__ __forceinline__ CFs cfs_add(CFs a, float b) {
    const float t = a.s + b;
    const float bb = t - a.s;
    const float err = (a.s - (t - bb)) + (b - bb);
    return CFs{t, a.c + err};
}
__device__ __forceinline__ CFs cfs_merge(CFs a, CFs b) {
    CFs r = cfs_add(a, b.s);
    r.c += b.c;
    return r;
}

template <int NC>
__global__ void __launch_bounds__(kObsThreads)
    k_obs_natural(const float* __restrict__ spins, int L, int chunks_per_rep, float J,
                  double* __restrict__ partials) {
    const int chunk = blockIdx.x;
    const int r = chunk / chunks_per_rep;
    const int64_t n = (int64_t)L * L * L;
    const int64_t start = (int64_t)(chunk - r * chunks_per_rep) * kObsChunk;
    const int64_t stop = start + kObsChunk < n ? start + kObsChunk : n;
    const float* S = spins + (int64_t)r * n * NC;
    CFs acc[kObsQ];
#pragma unroll
    for (int q = 0; q < kObsQ; ++q) acc[q] = CFs{0.f, 0.f};
    for (int64_t i = start + threadIdx.x; i < stop; i += blockDim.x) {
        const int x = (int)(i % L), y = (int)((i / L) % L), z = (int)(i / ((int64_t)L * L));
        const int64_t f[3] = {((int64_t)z * L + y) * L + (x + 1 == L ? 0 : x + 1),
                              ((int64_t)z * L + (y + 1 == L ? 0 : y + 1)) * L + x,
                              ((int64_t)(z + 1 == L ? 0 : z + 1) * L + y) * L + x};
        float s[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            s[c] = S[i * NC + c];
            acc[1 + c] = cfs_add(acc[1 + c], s[c]);
        }
        float e = 0.f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float* t = S + f[a] * NC;
            float d = 0.f;
#pragma unroll
            for (int c = 0; c < NC; ++c) d = fmaf(s[c], t[c], d);
            e += d;
            acc[4 + a] = cfs_add(acc[4 + a], d);
            acc[7 + a] = cfs_add(acc[7 + a], s[0] * t[1] - s[1] * t[0]);
        }
        acc[0] = cfs_add(acc[0], -J * e);
    }
    __shared__ CFs red[kObsThreads / 32][kObsQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kObsQ; ++q) {
        CFs v = acc[q];
        for (int o = 16; o > 0; o >>= 1) {
            CFs w{__shfl_down_sync(ISG_FULL_MASK, v.s, o), __shfl_down_sync(ISG_FULL_MASK, v.c, o)};
            v = cfs_merge(v, w);
        }
        if (lane == 0) red[wid][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < kObsQ) {
        CFs v = red[0][threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = cfs_merge(v, red[w][threadIdx.x]);
        partials[(int64_t)chunk * kObsQ + threadIdx.x] = (double)v.s + (double)v.c;
    }
}

__global__ void k_obs_combine(const double* __restrict__ partials, int replicas,
                              int chunks_per_rep, double* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= replicas) return;
    double q[kObsQ];
    for (int k = 0; k < kObsQ; ++k) q[k] = 0.0;
    for (int c = 0; c < chunks_per_rep; ++c)
        for (int k = 0; k < kObsQ; ++k)
            q[k] += partials[(int64_t)(r * chunks_per_rep + c) * kObsQ + k];
    for (int k = 0; k < kObsQ; ++k) out[(int64_t)r * kObsQ + k] = q[k];
}

std::mutex g_obs_mutex;
double* g_obs_ptr[kMaxDevices] = {};

}  // namespace
}  // namespace isg

extern "C" int isg_cont_observables_static(const float* d_spins, int L, int n_comp, int replicas,
                                           double J, double* d_out, void* stream) {
    using namespace isg;
    if (!d_spins || !d_out)
        return fail(ISG_ERR_ARG, "isg_cont_observables_static: NULL device pointer");
    if (n_comp != 2 && n_comp != 3)
        return fail(ISG_ERR_ARG, "isg_cont_observables_static: n_comp must be 2 or 3");
    if (L < 2 || replicas < 1)
        return fail(ISG_ERR_ARG, "isg_cont_observables_static: need L >= 2 and replicas >= 1");
    const int64_t n = (int64_t)L * L * L;
    const int64_t per_rep = (n + kObsChunk - 1) / kObsChunk;
    if (per_rep * replicas > kObsMaxChunks)
        return fail(ISG_ERR_ARG,
                    "isg_cont_observables_static: " + std::to_string(replicas) + " lattices of " +
                        std::to_string(L) + "^3 sites need " + std::to_string(per_rep * replicas) +
                        " partial blocks; the fixed scratch holds " +
                        std::to_string(kObsMaxChunks) + " (16,777,216 sites per call)");
    int dev = 0;
    ISG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(ISG_ERR_ARG, "isg_cont_observables_static: device ordinal out of range");
    double* scratch = nullptr;
    {
        // First call on a device: resolve the device address of the file-scope
        // scratch array (the host-side name is not a device address).
        std::lock_guard<std::mutex> lock(g_obs_mutex);
        if (!g_obs_ptr[dev]) {
            void* p = nullptr;
            ISG_CK(cudaGetSymbolAddress(&p, g_obs_partials));
            g_obs_ptr[dev] = static_cast<double*>(p);
        }
        scratch = g_obs_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = (int)(per_rep * replicas);
    if (n_comp == 3)
        k_obs_natural<3><<<blocks, kObsThreads, 0, st>>>(d_spins, L, (int)per_rep, (float)J,
                                                         scratch);
    else
        k_obs_natural<2><<<blocks, kObsThreads, 0, st>>>(d_spins, L, (int)per_rep, (float)J,
                                                         scratch);
    k_obs_combine<<<(replicas + 127) / 128, 128, 0, st>>>(scratch, replicas, (int)per_rep, d_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "isg_cont_observables_static launch");
    return ISG_OK;
}
