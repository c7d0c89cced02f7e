/*
 * isg.h — C ABI of libisinggb, the GB300 (sm_103a) checkerboard Monte Carlo
 * parallel-tempering engine for periodic cubic (and square) lattices.
 *
 * This is the drop-in boundary for the GPU backend of faulknco/ising-rs
 * (the Rust modules of src/cuda/ and src/parallel_tempering.rs).  Each entry point names the
 * reference interface it replaces.  Conventions:
 *
 *   - Every function returns an int status: ISG_OK (0) or a negative ISG_ERR_*
 *     code; isg_last_error() returns a thread-local text for the last failure.
 *     (Reference: anyhow::Result everywhere, e.g. src/cuda/lattice_gpu.rs:22,85.)
 *   - Host arrays are caller-owned; device memory is owned by the handle and is
 *     released by the matching *_destroy (reference: RAII CudaSlice,
 *     src/cuda/lattice_gpu.rs:9-19).
 *   - A handle is not thread-safe; all of its work is ordered on one CUDA
 *     stream (its own, or the caller's via *_set_stream).
 *   - Replica order in every per-replica array is size-major: index
 *     s*replicas + r for size index s and replica r.
 *
 * Random numbers (one definition shared by the kernels and any replay):
 *   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), key = {lo32(seed),
 *   hi32(seed)}, counter = {c0, c1, c2, c3} with
 *     c0 = stream uid: (L << 16) | replica  for a lattice replica,
 *                      (L << 16) | 0xFFFF   for the exchange stream of size L,
 *     c1 = index (per tag below),
 *     c2 = lo32(step),
 *     c3 = (tag << 24) | (colour << 16) | (hi32(step) & 0xFFFF).
 *   Only c1 varies across a warp, so the first rounds of every block are
 *   largely warp-uniform and are computed once per replica.
 */
#ifndef ISG_H
#define ISG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ISG_VERSION 100

#define ISG_OK               0
#define ISG_ERR_ARG         -1  /* bad argument (size, count, pointer)             */
#define ISG_ERR_CUDA        -2  /* a CUDA runtime call failed                       */
#define ISG_ERR_TIMEOUT     -3  /* a bounded device-side wait gave up               */
#define ISG_ERR_UNSUPPORTED -4  /* e.g. odd lattice size (no checkerboard under PBC) */
#define ISG_ERR_STATE       -5  /* call order (temperatures not set, ...)           */

/* Philox stream tags (c3 bits 24..31).
 *  INIT : hot start.  c1 = natural site index / 4, step = 0; word (site & 3);
 *         spin = -1 if the word's top bit is set, else +1.
 *  ISING: Metropolis half-sweep, step = global sweep number, colour = 0
 *         (x+y+z even) or 1.  A site of colour index i = (z*L*L + y*L + x) >> 1
 *         (2D: (y*L + x) >> 1) flips iff the 32-bit u = coarse << 25 | fine
 *         satisfies u <= threshold[own_down*8 + n_down_neighbours], with
 *         threshold = 0xFFFFFFFF for dE <= 0, else
 *         max(floor(exp(-beta*dE) * 2^32), 1) - 1  (FP64 on the host).
 *         With S = L^(dim-1)/2 sites of one colour per z-plane (3D) or row
 *         (2D), t = i / S, v = (t >> 2)*S + i % S:
 *           coarse = the low 7 bits of byte (v & 3) of word (t & 3) of the
 *                    block c1 = v >> 2, so one block serves 16 sites: 4 at
 *                    each of z (or y) = 4k .. 4k+3;
 *           fine   = bits 7..31 of word (i & 3) of the block
 *                    c1 = 0x80000000 | (i >> 2); it only matters when
 *                    coarse equals the threshold's top 7 bits.
 *  EXCH : replica exchange.  c1 = lower temperature index of the pair,
 *         c0 = exchange uid, step = exchange count of that size;
 *         u = ((w0 << 32 | w1) >> 11) * 2^-53.
 *  CINIT/CMETRO: continuous spins, c1 = natural site index (CINIT, one call
 *         per site) or colour index i (CMETRO: O(3) one call per site, words
 *         0..2; O(2) one call per index pair at c1 = i >> 1, words 0 and 2 for
 *         even i, 1 and 3 for odd i).
 */
#define ISG_TAG_INIT   0x01u
#define ISG_TAG_ISING  0x02u
#define ISG_TAG_EXCH   0x03u
#define ISG_TAG_CINIT  0x04u
#define ISG_TAG_CMETRO 0x05u
/* GRAPH: Ising on a graph (isg_graph_*).  c0 = replica, c1 = node / 4, word
 *        (node & 3), step = global sweep, colour field = colour class of the
 *        node (0xFE with step 0: hot start, spin -1 iff the top bit is set);
 *        flip iff u <= threshold[own_down][degree][n_down_neighbours].
 *        Exchanges use the EXCH tag with c0 = 0xFFFFFFFF. */
#define ISG_TAG_GRAPH  0x07u
/* CGRAPH: continuous spins on a graph (isg_cgraph_*).  c0 = replica,
 *        step = global sweep; field (colour bits) and c1:
 *          0xFE, c1 = node, step 0: hot start, O(3) z = 2 u0 - 1,
 *                phi = 2 pi u1; O(2) phi = 2 pi u0;
 *          class c, c1 = node: O(3) cone Metropolis, cos(theta) =
 *                1 - u0 (1 - cos delta), phi = 2 pi u1, accept iff dE <= 0
 *                or u2 < exp(-beta dE);
 *          0xFD, c1 = 0xFFFFFFFF: O(2) Wolff mirror angle 2 pi u0 and seed
 *                node (w1 * n) >> 32;
 *          0xC0 + k/4, c1 = node i, word k % 4: O(2) bond test of adjacency
 *                slot k of i, bond iff same-sign projections and
 *                u < 1 - exp(-2 beta J |p_i| |p_j|).
 *        u = 24-bit uniforms (w >> 8) 2^-24. */
#define ISG_TAG_CGRAPH 0x08u

const char* isg_last_error(void);
int isg_version(void);

/* ------------------------------------------------------------------------ */
/* Ising batch: every lattice size of a run x `replicas` replicas, int8 spins */
/* ------------------------------------------------------------------------ */
typedef struct isg_ising isg_ising;

/* Replaces LatticeGpu::new(n, seed) (src/cuda/lattice_gpu.rs:22-65) for all
 * (size, replica) pairs of a run at once, and the replica set built in
 * run_ising_fss (src/bin/gpu_fss.rs:188-193).  dim = 3 (cubic, the reference
 * path) or 2 (square).  Sizes must be even and 2..1024.  Spins start hot from
 * the ISG_TAG_INIT stream (the reference draws them unseeded,
 * src/cuda/lattice_gpu.rs:38-40). */
int isg_ising_create(isg_ising** out, const int* sizes, int n_sizes, int replicas,
                     int dim, uint64_t seed);
int isg_ising_destroy(isg_ising* h);

/* Work on the caller's CUDA stream (a cudaStream_t passed as void*); NULL
 * restores the handle's own stream.  The caller's stream must stay valid
 * until it is replaced or the handle is destroyed (destroy then waits for the
 * whole device rather than for that stream). */
int isg_ising_set_stream(isg_ising* h, void* cuda_stream);

/* Temperature grid per size (temps[s*replicas + t], slot t), coupling J and
 * field h.  Replaces the beta/J/h arguments of LatticeGpu::step
 * (src/cuda/lattice_gpu.rs:85) and linspace_temperatures
 * (src/parallel_tempering.rs:39-46) output handling in gpu_fss.  Resets the
 * replica->temperature maps to the identity. */
int isg_ising_set_temperatures(isg_ising* h, const double* temps, double J, double hfield);

/* n_sweeps full sweeps (colour 0 then colour 1) of every replica at the
 * temperature its r2t slot names; asynchronous.  Replaces LatticeGpu::step /
 * warm_up (src/cuda/lattice_gpu.rs:85-107,184-189). */
int isg_ising_step(isg_ising* h, int64_t n_sweeps);

/* Exact integer observables of every replica, synchronous:
 * bond_sum = sum over bonds s_i s_j, magnetisation = sum s_i, so that
 * E = -J*bond_sum - h*magnetisation.  Replaces measure_gpu / energy_gpu
 * (src/cuda/lattice_gpu.rs:116-181; reduce_kernel.cu:7-66).  The energies
 * are kept on the device for isg_ising_exchange. */
int isg_ising_measure(isg_ising* h, int64_t* bond_sum, int64_t* magnetisation);

/* One even (parity 0) or odd (parity 1) replica-exchange pass per size using
 * the energies of the last measurement; swaps temperature labels only.
 * parity < 0 uses the size's exchange count.  accepted[s] (may be NULL)
 * receives the swaps accepted for size s.  Synchronous.  Replaces
 * replica_exchange (src/parallel_tempering.rs:5-36). */
int isg_ising_exchange(isg_ising* h, int parity, int64_t* accepted);

/* Replica -> temperature-slot map (size-major, values 0..replicas-1). */
int isg_ising_get_r2t(isg_ising* h, int32_t* r2t);
int isg_ising_set_r2t(isg_ising* h, const int32_t* r2t);

/* Natural-layout spins (idx = z*L*L + y*L + x) of one replica.  Replaces
 * LatticeGpu::get_spins (src/cuda/lattice_gpu.rs:110-112). */
int isg_ising_get_spins(isg_ising* h, int size_index, int replica, int8_t* out);
int isg_ising_set_spins(isg_ising* h, int size_index, int replica, const int8_t* in);

/* The same, device to device and asynchronous on the handle's stream: d_nat is
 * a device buffer of L^dim +-1 bytes in natural layout. */
int isg_ising_load_natural(isg_ising* h, int size_index, int replica, const int8_t* d_nat);
int isg_ising_store_natural(isg_ising* h, int size_index, int replica, int8_t* d_nat);
/* Every replica of one size: d_nat[r * N + i] (N = L^dim), in one call. */
int isg_ising_store_natural_all(isg_ising* h, int size_index, int8_t* d_nat);

/* Parallel-tempering sampling: n_sweeps sweeps continuing the sampling phase;
 * after sampling sweep k (0-based, counted since the last reset) the
 * observables are measured if (k+1) % measure_every == 0 and an exchange pass
 * runs if (k+1) % exchange_every == 0, parity = exchange count % 2; each
 * measured sweep appends, per replica in replica order, one record
 * (temperature slot, bond_sum, magnetisation).  Records fill the caller's
 * arrays (max_records rows of n_sizes*replicas entries each); *n_records
 * returns the rows written.  The sweep/measure/exchange cycle runs as a CUDA
 * graph.  With all three record pointers NULL the call is asynchronous and
 * the records stay in a device ring (the newest ring rows survive) for
 * isg_ising_read_records.  Replaces the sampling loop of run_ising_fss
 * (src/bin/gpu_fss.rs:235-286). */
int isg_ising_pt_run(isg_ising* h, int64_t n_sweeps, int exchange_every, int measure_every,
                     int32_t* tslot_rec, int64_t* bond_rec, int64_t* mag_rec,
                     int64_t max_records, int64_t* n_records);

/* A temperature schedule on every lattice of the batch: n_sweeps full sweeps,
 * sweep k at temperature temps[k] for all lattices (temps NULL: every lattice
 * at its current slot temperature), no exchange.  After sweep k with
 * measure_every > 0 and k % measure_every == measure_phase, one record row of
 * (bond_sum, magnetisation) per lattice (index s*replicas + r) is appended to
 * bond/mag (max_records rows; *n_records returns the rows written).  With
 * temps given, every slot holds temps[n_sweeps-1] afterwards.  Lattices of at
 * most 65536 sites per colour run the whole schedule in one launch, one
 * thread-block cluster per lattice; larger ones sweep with the half-sweep
 * kernels.  Same random stream and results as isg_ising_step.  Synchronous
 * when records are written.  Replaces the sweep-by-sweep temperature loops of
 * src/cuda/fss_gpu.rs:19-33, src/cuda/kz_gpu.rs:17-40 and
 * src/cuda/coarsening_gpu.rs:10-28 (LatticeGpu::step per sweep, with a
 * full spin copy per measurement). */
int isg_ising_run_schedule(isg_ising* h, const double* temps, int64_t n_sweeps, int measure_every,
                           int measure_phase, int64_t* bond_rec, int64_t* mag_rec,
                           int64_t max_records, int64_t* n_records);

/* Copy the records still held in the device ring (at most max_records, the
 * newest ones) to the caller's arrays; synchronous. */
int isg_ising_read_records(isg_ising* h, int32_t* tslot_rec, int64_t* bond_rec, int64_t* mag_rec,
                           int64_t max_records, int64_t* n_records);

/* Zero the sampling-phase counters (sampling sweep, exchange counts, accepted
 * counts); called between warmup and sampling. */
int isg_ising_reset_sampling(isg_ising* h);

/* Accepted swaps so far per size (sum over pairs). */
int isg_ising_get_accepted(isg_ising* h, int64_t* accepted);

/* Global sweep counter (warmup + sampling), the Philox step of ISG_TAG_ISING. */
int isg_ising_get_sweep(isg_ising* h, uint64_t* sweep);

int isg_ising_sync(isg_ising* h);

/* Launch shape of the half-sweep kernel: blocks per SM (0 = occupancy
 * maximum).  Every size, site-block tasks included, runs in the one 256-thread
 * half-sweep kernel, so `threads` (64, 128, 256 or 512) is validated and
 * kept but no longer changes the launch.  Results never depend on either. */
int isg_ising_set_launch(isg_ising* h, int threads, int blocks_per_sm);
/* Prefetch form of the rolling half-sweep (3D, L = 32..256): 1 = loads one
 * plane ahead into registers; 2 = two planes ahead; 3 = (four words per lane)
 * copies into a per-warp ring in shared memory, own words two planes and the
 * other colour three planes ahead; 0 = automatic (3 with four words per
 * lane, else 2 when all spin planes fit in 96 MiB, else 1; 3 falls back to
 * that choice with two words per lane).  Results never depend on it. */
int isg_ising_set_prefetch(isg_ising* h, int depth);
/* Rolling half-sweep (3D, L = 64..256): lanes of each warp also prefetch the
 * lines of the task's own and other-colour words (and halo rows) `planes`
 * z-planes ahead of the plane being updated into L1 (level 1) or L2 (level 2);
 * planes = 0 turns it off (at most 16).  Results never depend on it. */
int isg_ising_set_cache_prefetch(isg_ising* h, int level, int planes);
/* Words of 4 sites each lane of the rolling half-sweep updates per plane for
 * L >= 128: 4 (default; 128-bit loads and stores, 2 blocks per SM) or 2 (as
 * for L = 64).  Results never depend on it. */
int isg_ising_set_words_per_lane(isg_ising* h, int words);
/* Launch the half-sweep word kernels as programmatic dependent launches
 * (enable = 1, default): their blocks are scheduled while the previous kernel
 * of the stream drains and wait for it before reading any device state; 0 =
 * ordinary launches.  Results never depend on it. */
int isg_ising_set_dependent_launch(isg_ising* h, int enable);
/* isg_ising_pt_run with host record arrays on a batch of small lattices (at
 * most 16 x 1024 sites per colour plane, all resident at once, no energy
 * histograms): enable = 1 (default) runs the whole PT cycle — sweeps, fused
 * measurements, records and exchanges at a bounded grid barrier — in one
 * cooperative launch of the cluster-resident kernel per 65,536 sweeps; 0 =
 * the CUDA-graph cycle of separate launches.  Results are the same bit for
 * bit; a barrier wait that gives up returns ISG_ERR_TIMEOUT. */
int isg_ising_set_resident_pt(isg_ising* h, int enable);
/* Time every supported launch shape (prefetch depth x site-kernel threads x
 * blocks per SM) on a scratch copy of the lattices and keep the fastest.
 * best[0..2] (may be NULL) receives threads, blocks/SM, prefetch depth. */
int isg_ising_autotune(isg_ising* h, int* best);

/* Mean device time (ms, CUDA events on the handle's stream) of one half-sweep
 * launch over n_launches launches of the current batch (colours alternate). */
int isg_ising_time_halfsweep(isg_ising* h, int n_launches, float* avg_ms);
/* Mean device time (ms) of one half-sweep launch as it runs inside a PT cycle:
 * n_launches launches (1..4096, colours alternating) captured as one CUDA
 * graph, each of `replays` replays preceded by a write of flush_bytes of
 * scratch memory (0 = no flush), events around the graph alone.  Spins and
 * sweep counter are restored.  Measurement utility (no reference counterpart;
 * it backs the roofline figures of the bench). */
int isg_ising_time_halfsweep_graph(isg_ising* h, int n_launches, int64_t flush_bytes,
                                   int replays, float* avg_ms);

/* Sites updated by one half-sweep launch (all sizes and replicas). */
int isg_ising_sites_per_halfsweep(isg_ising* h, int64_t* sites);

/* ------------------------------------------------------------------------ */
/* Continuous spins: O(3) Heisenberg (n_comp 3) and O(2) XY (n_comp 2)        */
/* ------------------------------------------------------------------------ */
typedef struct isg_cont isg_cont;

/* Replaces ContinuousGpuLattice::new(n, n_comp, seed, device)
 * (src/cuda/gpu_lattice_continuous.rs:24-88) for every (size, replica) of a
 * run.  FP32 unit vectors start uniform on the sphere (O(3): z and phi
 * uniform) or at a uniform angle (O(2)) from the ISG_TAG_CINIT stream. */
int isg_cont_create(isg_cont** out, const int* sizes, int n_sizes, int replicas, int n_comp,
                    uint64_t seed);
int isg_cont_destroy(isg_cont* h);
int isg_cont_set_stream(isg_cont* h, void* cuda_stream);
/* Temperature grid per size (as isg_ising_set_temperatures) and coupling J. */
int isg_cont_set_temperatures(isg_cont* h, const double* temps, double J);

/* n_sweeps sweeps, each n_overrelax overrelaxation sweeps then one Metropolis
 * sweep (the reference GPU order, gpu_lattice_continuous.rs:112-173); the
 * Metropolis proposal rotates the spin uniformly inside a cone of half-angle
 * delta (O(2): angle step uniform in [-delta, delta]).  Replaces
 * ContinuousGpuLattice::sweep. */
int isg_cont_sweep(isg_cont* h, int64_t n_sweeps, double delta, int n_overrelax);
/* Single half-sweeps: overrelaxation (continuous_spin_kernel.cu:88-142) and
 * Metropolis (continuous_spin_kernel.cu:9-83) of one colour. */
int isg_cont_overrelax(isg_cont* h, int colour);
int isg_cont_metropolis(isg_cont* h, int colour, double delta);
/* Rescale every spin to unit length. */
int isg_cont_normalize(isg_cont* h);

/* Observables of every replica, synchronous: energy[r] = -J sum_bonds S.S',
 * mag[r*3 + k] = sum S_k (k = 2 is 0 for XY), bonds[r*6 + a] (may be NULL) =
 * sum_i S_i.S_{i+a} for a = x, y, z, then sum_i (S_i x S_{i+a})_z: the
 * helicity-modulus sums.  Exact fixed-point sums (each term rounded once to a
 * multiple of 2^-24, int64 across threads and blocks, one FP64 conversion):
 * the result does not depend on the order of summation.  Replaces ContinuousGpuLattice::measure_gpu
 * (gpu_lattice_continuous.rs:177-240; reduce_kernel.cu:70-151). */
int isg_cont_measure(isg_cont* h, double* energy, double* mag, double* bonds);
/* Exchange pass on the energies of the last measurement (as
 * isg_ising_exchange; src/parallel_tempering.rs:5-36). */
int isg_cont_exchange(isg_cont* h, int parity, int64_t* accepted);
int isg_cont_reset_sampling(isg_cont* h);

/* PT sampling as isg_ising_pt_run, with renormalisation of every spin on
 * sweeps k where (global sweep + 1) % renorm_every == 0 (0 = never).
 * Records: slot, energy, mag[3], bonds[6] per replica per measured sweep.
 * Replaces the sampling loop of run_continuous_fss (gpu_fss.rs:494-545). */
int isg_cont_pt_run(isg_cont* h, int64_t n_sweeps, int exchange_every, int measure_every,
                    double delta, int n_overrelax, int renorm_every, int32_t* tslot_rec,
                    double* energy_rec, double* mag_rec, double* bonds_rec, int64_t max_records,
                    int64_t* n_records);
int isg_cont_get_r2t(isg_cont* h, int32_t* r2t);
/* Natural-layout spins, n_comp floats per site interleaved as the reference
 * stores them (continuous_spin_kernel.cu:6). */
int isg_cont_get_spins(isg_cont* h, int size_index, int replica, float* out);
int isg_cont_set_spins(isg_cont* h, int size_index, int replica, const float* in);
/* Exchange swaps accepted per size; Metropolis moves accepted per replica. */
int isg_cont_get_accepted(isg_cont* h, int64_t* accepted);
int isg_cont_get_metro_accepted(isg_cont* h, int64_t* accepted);
int isg_cont_sync(isg_cont* h);
/* Mean device ms of one overrelaxation half-sweep, one Metropolis half-sweep,
 * one measurement and one colour-1 Metropolis half-sweep with the measurement
 * fused in (0 when the batch runs the one-site kernels) (out[4]); the
 * lattices are restored afterwards. */
int isg_cont_time_kernels(isg_cont* h, int n, float* out_ms);
/* Measured sweeps of isg_cont_pt_run: 1 (default) fuses the measurement into
 * the colour-1 Metropolis half-sweep when every size is a multiple of 4 (one
 * pass over the lattices less); 0 measures in a separate pass.  Results are
 * the same bit for bit. */
int isg_cont_set_fused_measure(isg_cont* h, int enable);
/* Site updates of one full sweep of one kind (all sizes and replicas). */
int isg_cont_sites_per_sweep(isg_cont* h, int64_t* sites);

/* Observables of continuous-spin lattices that the caller owns, computed
 * without any allocation by the library.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc (their device memory comes
 * from their own pool or framework, or allocation is not allowed where they
 * run).  d_spins: `replicas` lattices of L^3 sites in the reference's natural
 * interleaved layout (n_comp floats per site, site z*L*L + y*L + x), device
 * memory; d_out: device memory for replicas*10 doubles, per replica E, Mx, My,
 * Mz, then sum_i S_i.S_{i+a} and sum_i (S_i x S_{i+a})_z for a = x, y, z (the
 * layout of isg_cont_measure).  Work is queued on `stream` (NULL = the legacy
 * default stream); the call does not synchronise.  Block partials live in a
 * fixed device array of 16384 blocks of 1024 sites (replicas * ceil(L^3/1024)
 * must not exceed 16384, i.e. at most 16,777,216 sites per call; larger
 * requests return ISG_ERR_ARG).  The first call on each device looks up that
 * array's device address, so make it before capturing a stream into a graph.
 * That address is kept for the life of the process: after cudaDeviceReset (or
 * anything else that tears down the device's primary context and reloads the
 * module) it is stale, so do not use this entry point again in that process.
 * All calls share the array: calls that overlap on the GPU (different
 * streams, no ordering) race and must be serialised by the caller. */
int isg_cont_observables_static(const float* d_spins, int L, int n_comp, int replicas, double J,
                                double* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Learned autoregressive proposal (no reference counterpart)                 */
/* ------------------------------------------------------------------------ */
/* A masked-convolution autoregressive network over an H x W raster of +-1
 * spins (a cubic L^3 lattice is the L^2 x L raster of its z-y rows): layers
 * 3x3 mask A (1 -> 32), then mask B (32 -> 32) ..., last mask B (32 -> 1
 * logit), ReLU, BF16 weights, FP32 accumulation.  q(s) = prod sigma(s_i l_i);
 * proposals use q_sym(s) = (q(s) + q(-s)) / 2 and an exact independence
 * Metropolis-Hastings test.  Configuration buffers are natural-layout +-1
 * bytes.  All device work runs on the handle's stream (isg_learned_stream). */
typedef struct isg_learned isg_learned;
int isg_learned_create(isg_learned** out, int H, int W, int layers, uint64_t seed);
/* As isg_learned_create, for the raster of a 3D lattice: zrow = rows per
 * z-plane (L for the L^2 x L raster of an L^3 lattice; 0 = 2D).  Layer 0 then
 * has a fifth tap, the site one z-plane back (zrow rows up, same x), so the
 * network sees the z-neighbour that the 3x3 raster taps cannot reach. */
int isg_learned_create2(isg_learned** out, int H, int W, int zrow, int layers, uint64_t seed);
int isg_learned_destroy(isg_learned* h);
int isg_learned_num_params(isg_learned* h, int* n);
int isg_learned_get_weights(isg_learned* h, float* w);
int isg_learned_set_weights(isg_learned* h, const float* w);
/* Mean negative log-likelihood of B host configurations and its gradient. */
int isg_learned_gradient(isg_learned* h, const int8_t* cfg, int B, float* grad, float* nll);
/* `steps` Adam steps on batches of B taken cyclically from n device configurations. */
int isg_learned_train(isg_learned* h, const int8_t* d_cfg_all, int n, int B, int steps, float lr,
                      float* last_mean_logq);
/* K samples of q with log q, and log q of their negations (same kernel). */
int isg_learned_sample(isg_learned* h, int K, uint64_t step, int8_t* d_out, float* d_lq,
                       float* d_lq_flip);
/* Proposals per full wave of the sampling kernel on this device: batches of a
 * multiple of it leave no SM idle in the last wave. */
int isg_learned_batch_quantum(isg_learned* h, int* quantum);
/* log q of K device configurations (flip = 1: of their negations). */
int isg_learned_score(isg_learned* h, const int8_t* d_cfg, int K, int flip, float* d_lq);
/* Exact bond sums and magnetisations of K device configurations (L^dim, PBC). */
int isg_learned_energies(isg_learned* h, const int8_t* d_cfg, int K, int L, int dim,
                         int64_t* d_bond, int64_t* d_mag);
/* One independence MH pass over K proposals; see isg_learned.cu. */
int isg_learned_imh(isg_learned* h, const int64_t* d_bond, const int64_t* d_mag,
                    const float* d_lq, const float* d_lq_flip, int K, double beta, double J,
                    int64_t* d_state, double* d_ax, int64_t* d_mrec, int64_t* d_brec,
                    int64_t* d_accepted, double* d_work, uint64_t step);
/* A = -beta E - log q_sym of one configuration (device scalars). */
int isg_learned_state_a(isg_learned* h, const float* d_lq, const float* d_lq_flip,
                        const int64_t* d_bond, double beta, double J, double* d_ax);
/* Copy proposal d_state[2] (if >= 0) into the current configuration. */
int isg_learned_adopt(isg_learned* h, const int8_t* d_props, const int64_t* d_state,
                      int8_t* d_current);
int isg_learned_sync(isg_learned* h);
void* isg_learned_stream(isg_learned* h);

/* ------------------------------------------------------------------------ */
/* Annealing finite-size scaling (`fss --gpu`)                               */
/* ------------------------------------------------------------------------ */

/* Replaces run_fss_gpu (src/cuda/fss_gpu.rs:7-39) with LatticeGpu::warm_up
 * and LatticeGpu::measure (src/cuda/lattice_gpu.rs:184-251).  Every size is
 * one lattice, annealed from t_max down to t_min through the t_steps
 * temperatures T_k = t_min + (t_max - t_min)*k/(t_steps - 1): at each one,
 * `warmup` sweeps, then `samples` sweeps each followed by a measurement of E
 * and M (fused into the sweep; no spin copies).  out[(i*t_steps + k)*7 + j]
 * receives for sizes[i], in ascending temperature order k, the Observables
 * fields (src/observables.rs:5-13) j = 0..6: T, <e>, <|m|>, <m^2>, <m^4>,
 * Cv = beta^2 (<e^2> - <e>^2) N, chi = beta (<m_s^2> - <m_s>^2) N with the
 * signed m_s (lattice_gpu.rs:236-240), summed in sample order in FP64.
 * All sizes run in one batch (one replica each); the stream of size L is
 * keyed by (seed, L), where the reference seeds size n with seed + n
 * (fss_gpu.rs:13).  Thresholds use beta = 1/T in FP64 (the reference passes
 * an f32 beta to the kernel).  A repeated size repeats its rows.  Synchronous;
 * creates and destroys its own batch. */
int isg_fss_anneal(const int* sizes, int n_sizes, int dim, double t_min, double t_max,
                   int t_steps, double J, double hfield, int64_t warmup, int64_t samples,
                   uint64_t seed, double* out);

/* ------------------------------------------------------------------------ */
/* Quench protocols (`kz --gpu`, `coarsening --gpu`)                         */
/* ------------------------------------------------------------------------ */

/* Replaces run_kz_sweep_gpu / run_kz_gpu (src/cuda/kz_gpu.rs:9-95) on a cubic
 * n^3 lattice: for every tau_q[i], n_trials lattices are warmed up for
 * warmup_sweeps sweeps at t_start, ramped linearly over tau_q[i] sweeps
 * (sweep k at max(t_start + (t_end - t_start)*(k+1)/tau_q, 0.01),
 * kibble_zurek.rs:78-84), then held freeze_sweeps sweeps at
 * max(freeze_temperature, 0.01); the final domain-wall density
 * rho = walls / (3 n^3) over the forward bonds (lattice_gpu.rs:253-281) gives
 * out[2*i] = mean and out[2*i+1] = standard error over the trials
 * (mean_and_std_err, kibble_zurek.rs:86-100).  Trial t of tau_q uses replica
 * t of a batch keyed by base_seed + tau_q (the reference seeds it with
 * base_seed + tau_q + t).  All tau_q values run concurrently, each schedule
 * in one launch for n^3 <= 131072.  Synchronous. */
int isg_kz_sweep(int n, double J, double t_start, double t_end, const int64_t* tau_q, int n_tau,
                 int n_trials, int64_t warmup_sweeps, int64_t freeze_sweeps,
                 double freeze_temperature, uint64_t base_seed, double* out);

/* Replaces run_coarsening_gpu (src/cuda/coarsening_gpu.rs:6-31) on a cubic
 * n^3 lattice: warmup_sweeps sweeps at t_high, then total_steps sweeps at
 * max(t_quench, 0.01); after sweep `step` with step % sample_every == 0 the
 * point (step, rho) is written to steps_out / rho_out (max_points entries,
 * *n_points returns the count), rho being the domain-wall density of the
 * forward bonds from the fused bond sum.  Synchronous. */
int isg_coarsening(int n, double J, double t_high, double t_quench, int64_t warmup_sweeps,
                   int64_t total_steps, int64_t sample_every, uint64_t seed, int64_t* steps_out,
                   double* rho_out, int64_t max_points, int64_t* n_points);

/* ------------------------------------------------------------------------ */
/* Ising parallel tempering on graphs (`gpu_jfit --model ising`)             */
/* ------------------------------------------------------------------------ */
typedef struct isg_graph isg_graph;

/* Replaces the replica set of run_ising_jfit (src/bin/gpu_jfit.rs:172-213) on
 * a graph given as an edge list (GraphDef, src/graph.rs:4-79): edges[2e],
 * edges[2e+1] are the ends of edge e (no self-loops, degree at most 12,
 * n_nodes <= 65536).  `replicas` copies start hot from the GRAPH stream.
 * Sites are updated colour class by colour class of a greedy proper colouring
 * (node order; isg_graph_num_colours), one CTA per replica. */
int isg_graph_create(isg_graph** out, int n_nodes, const int32_t* edges, int n_edges,
                     int replicas, uint64_t seed);
int isg_graph_destroy(isg_graph* h);
int isg_graph_num_colours(isg_graph* h, int* n_colours);
/* Temperature of slot t (temps[t], `replicas` entries) and coupling J; resets
 * the replica <-> temperature maps to the identity. */
int isg_graph_set_temperatures(isg_graph* h, const double* temps, double J);
/* Warm-up sweeps (no measurement, no exchange). */
int isg_graph_step(isg_graph* h, int64_t n_sweeps);
int isg_graph_reset_sampling(isg_graph* h);
/* Sampling as isg_ising_pt_run: after sampling sweep k, records (slot, bond
 * sum, magnetisation) per replica if (k+1) % measure_every == 0, and an
 * exchange pass (src/parallel_tempering.rs:5-36, energies E = -J * bond of the
 * last sweep, parity = exchange count % 2) if (k+1) % exchange_every == 0.
 * Replaces the sampling loop of run_ising_jfit (gpu_jfit.rs:225-262).
 * Synchronous. */
int isg_graph_pt_run(isg_graph* h, int64_t n_sweeps, int exchange_every, int measure_every,
                     int32_t* tslot_rec, int64_t* bond_rec, int64_t* mag_rec,
                     int64_t max_records, int64_t* n_records);
int isg_graph_get_accepted(isg_graph* h, int64_t* accepted);
int isg_graph_get_spins(isg_graph* h, int replica, int8_t* out);
int isg_graph_get_r2t(isg_graph* h, int32_t* r2t);
/* When all replicas fit on the GPU at once (and exchange_every <= 100000),
 * isg_graph_pt_run and isg_cgraph_pt_run run as one cooperative launch whose
 * replicas meet at a grid barrier at every exchange point.  Every wait there is
 * bounded (about 8 s of clock cycles); when one runs out the call returns
 * ISG_ERR_TIMEOUT and the handle's state is undefined (destroy it).
 * isg_barrier_selftest launches `blocks` blocks that wait at
 * that barrier for `expected` arrivals with a limit of `limit_cycles`:
 * *timed_out = 1 when the waits ran out (expected > blocks), else 0. */
int isg_barrier_selftest(int blocks, int expected, int64_t limit_cycles, int* timed_out);

/* ------------------------------------------------------------------------ */
/* Continuous spins on graphs (`gpu_jfit --model heisenberg|xy`)             */
/* ------------------------------------------------------------------------ */
typedef struct isg_cgraph isg_cgraph;

/* Replaces the replica sets of run_heisenberg_jfit (n_comp = 3,
 * src/bin/gpu_jfit.rs:414-447) and run_xy_jfit (n_comp = 2,
 * gpu_jfit.rs:299-330): `replicas` copies of a graph (edge list as
 * isg_graph_create; degree at most 64, n_nodes <= 16384) with FP32 unit spins,
 * hot from the CGRAPH stream.  One CTA per replica holds its spins in shared
 * memory.  O(3) sweeps are cone Metropolis (half-angle isg_cgraph_set_delta,
 * default 0.5 as gpu_jfit.rs:450) by colour class of a greedy proper
 * colouring; an O(2) sweep is one single-cluster Wolff flip
 * (src/xy/wolff.rs:15-78) grown breadth-first by the CTA. */
int isg_cgraph_create(isg_cgraph** out, int n_nodes, const int32_t* edges, int n_edges,
                      int replicas, int n_comp, uint64_t seed);
int isg_cgraph_destroy(isg_cgraph* h);
int isg_cgraph_num_colours(isg_cgraph* h, int* n_colours);
/* Temperature of slot t and coupling J; resets the ladder to the identity. */
int isg_cgraph_set_temperatures(isg_cgraph* h, const double* temps, double J);
int isg_cgraph_set_delta(isg_cgraph* h, double delta);
int isg_cgraph_step(isg_cgraph* h, int64_t n_sweeps);
int isg_cgraph_reset_sampling(isg_cgraph* h);
/* As isg_graph_pt_run with per-record energy E = -J sum_bonds S.S' (FP64 sum
 * of FP32 node terms) and magnetisation vector m_rec[(row*R + r)*n_comp + k];
 * replaces the sampling loops of gpu_jfit.rs:349-377 and 462-490. */
int isg_cgraph_pt_run(isg_cgraph* h, int64_t n_sweeps, int exchange_every, int measure_every,
                      int32_t* tslot_rec, double* e_rec, double* m_rec, int64_t max_records,
                      int64_t* n_records);
int isg_cgraph_get_accepted(isg_cgraph* h, int64_t* accepted);
/* Per replica since the last reset: accepted rotations (O(3)) or the summed
 * cluster sizes (O(2)). */
int isg_cgraph_get_moves(isg_cgraph* h, int64_t* moves);
/* Spins of one replica, natural layout out[node*n_comp + k]. */
int isg_cgraph_get_spins(isg_cgraph* h, int replica, float* out);
int isg_cgraph_set_spins(isg_cgraph* h, int replica, const float* in);
int isg_cgraph_get_r2t(isg_cgraph* h, int32_t* r2t);
int isg_cgraph_get_sweep(isg_cgraph* h, uint64_t* sweep);

/* ------------------------------------------------------------------------ */
/* Energy histograms and reweighting (the consumers of the PT timeseries)    */
/* ------------------------------------------------------------------------ */

/* Device energy histograms of an Ising batch, accumulated by every record of
 * isg_ising_pt_run (not by isg_ising_run_schedule): per size and temperature
 * slot, exact bins of the bond sum B (bin b holds B = 4 b - dN, d = dim,
 * N = L^d; B + dN is always a multiple of 4 on a periodic even lattice), each
 * with 4 uint64 counters: samples, and the sums of |m|, m^2, m^4 (m = M / N) in
 * units of 2^-32 (each term rounded to nearest).  With h = 0 the energy of a bin
 * is E = -J B, so histogram reweighting in temperature is exact.  Replaces the
 * per-sample (E, |m|) timeseries that analysis/scripts/analyze_gpu_fss.py:60-83
 * reads for reweighting.  Full-range bins: dN/2 + 1 per slot, 32 bytes each.
 * enable = 0 frees them; enabling again clears them. */
int isg_ising_hist_enable(isg_ising* h, int enable);
int isg_ising_hist_reset(isg_ising* h);
/* Visited bins of (size, slot): *bond_lo = B of the lowest, *n_bins = number
 * from the lowest to the highest (0 if no record yet). */
int isg_ising_hist_range(isg_ising* h, int size_index, int slot, int64_t* bond_lo,
                         int64_t* n_bins);
/* out[4*i + {0..3}] = counters of the bin with B = bond_lo + 4 i. */
int isg_ising_hist_read(isg_ising* h, int size_index, int slot, int64_t bond_lo, int64_t n_bins,
                        uint64_t* out);

/* Multiple-histogram (WHAM) reweighting, analysis/scripts/reweighting.py:45-105
 * and analyze_gpu_fss.py:160-243, on the GPU in FP64.  P points: energy e[p]
 * (total), weight c[p] (1 for a sample, the count of a histogram bin), moment
 * sums mom[p*n_mom + j] (n_mom <= 8; e.g. the point's sums of |m|, m^2, m^4).
 * K simulations: beta[k], sample counts n_k[k].  The free energies f_k
 * (f_0 = 0) iterate as the reference does (at most n_iter rounds, stop when
 * max |f' - f| < tol; the weights use the last round's denominators).  For T
 * targets beta_t: out[t*(3+n_mom) + {0, 1, 2, 3+j}] = log Z, <E>, <E^2>, <mom_j>
 * with <mom_j> = sum_p w_p mom_pj / sum_p w_p c_p.  f_out[K], iters_out may be
 * NULL. */
int isg_wham(const double* e, const double* c, const double* mom, int n_mom, int64_t P,
             const double* beta, const double* n_k, int K, int n_iter, double tol,
             const double* beta_t, int T, double* out, double* f_out, int* iters_out);
/* The reference's normalised per-point weights at one target (wham_reweight's
 * w): w[p] = c_p exp(-beta_t E_p - log_denom_p) / Z. */
int isg_wham_weights(const double* e, const double* c, int64_t P, const double* beta,
                     const double* n_k, int K, int n_iter, double tol, double beta_t, double* w,
                     double* f_out, int* iters_out);
/* Single-histogram reweighting (reweighting.py:15-43, analyze_gpu_fss.py:86-157):
 * target t reweights the points [p0[t], p1[t]) of the simulation at beta_ref[t],
 * leaving out [x0[t], x1[t]) (x0 = x1 = NULL: none; a jackknife block), by
 * exp(-(beta_t - beta_ref) E); out as isg_wham. */
int isg_reweight_single(const double* e, const double* c, const double* mom, int n_mom, int64_t P,
                        const int64_t* p0, const int64_t* p1, const int64_t* x0, const int64_t* x1,
                        const double* beta_ref, const double* beta_t, int T, double* out);

/* Binary timeseries file (the compact form of gpu_fss_{model}_N{n}_timeseries.csv,
 * src/bin/gpu_fss.rs:212-290), little-endian:
 *   char magic[8] = "ISGTSER1"; uint32 header_bytes = 32 + 8 n_temps;
 *   uint32 model (0 ising, 1 heisenberg, 2 xy); uint32 n; uint32 n_temps;
 *   uint64 reserved = 0; double temps[n_temps];
 *   then records to the end of the file, 24 bytes each:
 *   uint32 temp_idx; uint32 replica; double E (per spin); double M (|m| per spin).
 * Host-only calls (no device work). */
typedef struct isg_ts isg_ts;
int isg_ts_open(isg_ts** out, const char* path, int model, int n, const double* temps,
                int n_temps);
int isg_ts_append(isg_ts* f, const int32_t* temp_idx, const int32_t* replica, const double* e,
                  const double* m, int64_t count);
int isg_ts_close(isg_ts* f);
/* Histogram file (gpu_fss_ising_N{n}_hist.bin), little-endian:
 *   char magic[8] = "ISGHIST1"; uint32 header_bytes = 32 + 8 n_temps;
 *   uint32 dim; uint32 n; uint32 n_temps; double J; double temps[n_temps];
 *   then per temperature: int64 bond_lo; int64 n_bins; n_bins x 4 uint64
 *   (the isg_ising_hist_read counters).  counters holds the temperatures'
 *   blocks one after another. */
int isg_hist_write(const char* path, int dim, int n, double J, const double* temps, int n_temps,
                   const int64_t* bond_lo, const int64_t* n_bins, const uint64_t* counters);

/* ------------------------------------------------------------------------ */
/* Statistics used by the drop-in driver                                     */
/* ------------------------------------------------------------------------ */

/* Leave-one-block-out jackknife of a (e, m) series exactly as
 * jackknife_observables (src/bin/gpu_fss.rs:327-412).  out[12] =
 * E, E_err, M, M_err, M2, M2_err, M4, M4_err, Cv, Cv_err, chi, chi_err. */
int isg_jackknife(const double* e, const double* m, int64_t n, double beta, double n_sites,
                  int n_blocks, double* out);

#ifdef __cplusplus
}
#endif
#endif /* ISG_H */
