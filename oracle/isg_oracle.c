/*
 * isg_oracle.c — CPU ORACLE for the checkerboard parallel-tempering path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libisinggb, gpu_fss, the
 * Python package) links, loads or calls this file; only tests/, the smoke
 * check and bench.py's CPU-baseline leg do, as the checker or the timed
 * reference-CPU baseline.
 *
 * Contents
 *  1. Philox4x32-10, restated from Salmon, Moraes, Dror & Shaw, "Parallel
 *     random numbers: as easy as 1, 2, 3" (SC'11): 10 rounds, multipliers
 *     0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85.
 *     Pinned on the GPU against curand's curand_Philox4x32_10 (called, not
 *     copied) by tests/test_gpu_ising.py.
 *  2. Checkerboard replay of the Ising update rule and random stream that the
 *     GPU path defines (include/isg.h): bit-exact oracle for spins and for the
 *     integer bond sum / magnetisation.  Physics of one update follows the
 *     reference kernel src/cuda/kernels.cu:33-55 (dE = 2 s (J nb + h),
 *     accept dE < 0 or u < exp(-beta dE)) with a uint32 threshold in place of
 *     the FP32 expf compare.
 *  3. Energy / magnetisation as src/observables.rs:165-181 (bond form of
 *     src/cuda/reduce_kernel.cu:27-66), returned as exact integers.
 *  4. Replica exchange as src/parallel_tempering.rs:5-36 (pairs from
 *     even_odd % 2, delta = (b_i - b_j)(E_j - E_i), accept delta < 0 or
 *     u < exp(-delta)) with u from the ISG_TAG_EXCH Philox stream in place of
 *     the host Xoshiro256++ (src/bin/gpu_fss.rs:197).
 *  5. The full PT protocol of run_ising_fss (src/bin/gpu_fss.rs:186-286):
 *     warmup, then sweep / measure / exchange with (k+1) % every cadence.
 *  6. The reference CPU Metropolis path (src/metropolis.rs:8-27 random-site
 *     sweep, src/lattice.rs:132-151 cubic neighbours, src/lattice.rs:85-100
 *     square neighbours, src/lattice.rs:73-77 randomise), driven by
 *     Xoshiro256++ seeded through SplitMix64 as rand_xoshiro 0.6.0
 *     Xoshiro256PlusPlus::seed_from_u64 does, with rand 0.8.5's
 *     gen_range (widening multiply + zone rejection), gen::<f64>
 *     ((x >> 11) * 2^-53) and gen_bool(0.5) (x < 2^63) restated from their
 *     published algorithms (neither crate is vendored in the reference).
 *     This is the timed "reference CPU path" baseline; it is statistical
 *     only (no reference test pins a stream value).
 *  7. Jackknife exactly as src/bin/gpu_fss.rs:327-412.
 *
 * Parity pinning: the Philox restatement is pinned against curand on the GPU;
 * the physics is pinned statistically against the reference's committed PT
 * summaries (analysis/data/gpu_windows_pipeline/publication/ summary CSVs, fixtures
 * in tests/golden/) and against exact enumeration.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, so that FP64 sums round
 * exactly as the device code's explicit _rn operations do).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>

/* ------------------------------------------------------------------ 1 */
#define PH_M0 0xD2511F53u
#define PH_M1 0xCD9E8D57u
#define PH_W0 0x9E3779B9u
#define PH_W1 0xBB67AE85u

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PH_M0 * c0;
        uint64_t p1 = (uint64_t)PH_M1 * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += PH_W0;
        k1 += PH_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define TAG_INIT 0x01u
#define TAG_ISING 0x02u
#define TAG_EXCH 0x03u
#define TAG_CINIT 0x04u
#define TAG_CMETRO 0x05u

/* counter = {stream uid, index, lo32(step), tag | colour | hi16(step)} */
static void stream_words(uint64_t seed, uint32_t index, uint32_t uid, uint64_t step, uint32_t tag,
                         uint32_t colour, uint32_t out[4]) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {uid, index, (uint32_t)step,
                       (tag << 24) | (colour << 16) | ((uint32_t)(step >> 32) & 0xFFFFu)};
    or_philox4x32_10(ctr, key, out);
}

uint32_t or_replica_uid(int L, int r) { return ((uint32_t)L << 16) | (uint32_t)r; }
uint32_t or_exchange_uid(int L) { return ((uint32_t)L << 16) | 0xFFFFu; }

/* ------------------------------------------------------------------ 2 */
static int64_t nsites(int L, int dim) {
    return dim == 3 ? (int64_t)L * L * L : (int64_t)L * L;
}

/* thr[own_down*8 + n_down], accept iff u <= thr. */
void or_ising_thresholds(int dim, double beta, double J, double h, uint32_t thr[16]) {
    for (int i = 0; i < 16; ++i) thr[i] = 0;
    for (int od = 0; od < 2; ++od) {
        double s = od ? -1.0 : 1.0;
        for (int nd = 0; nd <= 2 * dim; ++nd) {
            double nb = (double)(2 * dim - 2 * nd);
            double dE = 2.0 * s * (J * nb + h);
            uint32_t t;
            if (dE <= 0.0) {
                t = 0xFFFFFFFFu;
            } else {
                double p = exp(-beta * dE);
                double f = floor(p * 4294967296.0);
                if (f < 1.0) f = 1.0;
                t = (uint32_t)(f - 1.0);
            }
            thr[od * 8 + nd] = t;
        }
    }
}

void or_ising_hot_start(int L, int dim, uint64_t seed, uint32_t uid, int8_t* spins) {
    int64_t n = nsites(L, dim);
    uint32_t w[4];
    for (int64_t i = 0; i < n; ++i) {
        if ((i & 3) == 0) stream_words(seed, (uint32_t)(i >> 2), uid, 0, TAG_INIT, 0, w);
        spins[i] = (w[i & 3] >> 31) ? -1 : 1;
    }
}

static inline int64_t site_index(int L, int dim, int x, int y, int z) {
    return dim == 3 ? ((int64_t)z * L + y) * L + x : (int64_t)y * L + x;
}

/* One colour of a checkerboard sweep on natural-layout spins.
 *
 * The 32-bit random u of a site at colour index ci = natural index >> 1 is
 * assembled from two Philox blocks of the ISING stream (the GPU kernels'
 * definition, include/isg.h):
 *   S = L^(dim-1)/2 sites of one colour per z-plane (3D) or row (2D),
 *   t = ci / S, j = ci % S, v = (t >> 2) * S + j;
 *   coarse = the low 7 bits of byte (v & 3) of word (t & 3) of block
 *            c1 = v >> 2 (one block serves the 16 sites of 4 slabs);
 *   fine   = bits 7..31 of word (ci & 3) of block c1 = 0x80000000 | (ci >> 2);
 *   u = coarse << 25 | fine, and the site flips iff u <= thr.
 * The fine block is only drawn when coarse equals thr's top 7 bits (otherwise
 * the comparison is already decided). */
void or_ising_halfsweep(int L, int dim, int8_t* spins, int colour, uint64_t seed, uint32_t uid,
                        uint64_t sweep, const uint32_t thr[16]) {
    int zmax = dim == 3 ? L : 1;
    const int64_t S = (dim == 3 ? (int64_t)L * L : (int64_t)L) / 2;
    uint32_t w[4], fw[4];
    int64_t cached_block = -1;
    for (int z = 0; z < zmax; ++z)
        for (int y = 0; y < L; ++y)
            for (int x = 0; x < L; ++x) {
                if (((x + y + z) & 1) != colour) continue;
                int64_t idx = site_index(L, dim, x, y, z);
                int64_t ci = idx >> 1;
                int xp = (x + 1) % L, xm = (x + L - 1) % L;
                int yp = (y + 1) % L, ym = (y + L - 1) % L;
                int nd = 0;
                nd += spins[site_index(L, dim, xp, y, z)] < 0;
                nd += spins[site_index(L, dim, xm, y, z)] < 0;
                nd += spins[site_index(L, dim, x, yp, z)] < 0;
                nd += spins[site_index(L, dim, x, ym, z)] < 0;
                if (dim == 3) {
                    int zp = (z + 1) % L, zm = (z + L - 1) % L;
                    nd += spins[site_index(L, dim, x, y, zp)] < 0;
                    nd += spins[site_index(L, dim, x, y, zm)] < 0;
                }
                int od = spins[idx] < 0;
                const uint32_t th = thr[od * 8 + nd];
                const int64_t t = ci / S, v = (t >> 2) * S + (ci - t * S);
                if ((v >> 2) != cached_block) {
                    cached_block = v >> 2;
                    stream_words(seed, (uint32_t)cached_block, uid, sweep, TAG_ISING,
                                 (uint32_t)colour, w);
                }
                const uint32_t coarse = (w[t & 3] >> (8 * (v & 3))) & 0x7Fu;
                int flip;
                if (coarse != (th >> 25)) {
                    flip = coarse < (th >> 25);
                } else {
                    stream_words(seed, 0x80000000u | (uint32_t)(ci >> 2), uid, sweep, TAG_ISING,
                                 (uint32_t)colour, fw);
                    flip = ((coarse << 25) | (fw[ci & 3] >> 7)) <= th;
                }
                if (flip) spins[idx] = (int8_t)(-spins[idx]);
            }
}

/* ------------------------------------------------------------------ 3 */
/* bond = sum over forward bonds s_i s_j (each of the 2*dim neighbour entries
 * of a site counted once per bond, as in observables.rs:165-181 with /2). */
void or_ising_measure(int L, int dim, const int8_t* spins, int64_t* bond, int64_t* mag) {
    int zmax = dim == 3 ? L : 1;
    int64_t b = 0, m = 0;
    for (int z = 0; z < zmax; ++z)
        for (int y = 0; y < L; ++y)
            for (int x = 0; x < L; ++x) {
                int64_t i = site_index(L, dim, x, y, z);
                int s = spins[i];
                m += s;
                b += s * spins[site_index(L, dim, (x + 1) % L, y, z)];
                b += s * spins[site_index(L, dim, x, (y + 1) % L, z)];
                if (dim == 3) b += s * spins[site_index(L, dim, x, y, (z + 1) % L)];
            }
    *bond = b;
    *mag = m;
}

/* ------------------------------------------------------------------ 4 */
static double u53(const uint32_t w[4]) {
    uint64_t x = ((uint64_t)w[0] << 32) | w[1];
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* energies indexed by replica; betas by temperature slot.  Returns accepted. */
int64_t or_exchange(int R, const double* betas, const double* energies, int32_t* r2t, int32_t* t2r,
                    int parity, uint64_t seed, uint32_t xuid, uint64_t xcount) {
    int64_t acc = 0;
    for (int i = parity & 1; i + 1 < R; i += 2) {
        int ri = t2r[i], rj = t2r[i + 1];
        double d = (betas[i] - betas[i + 1]) * (energies[rj] - energies[ri]);
        int ok = d < 0.0;
        if (!ok) {
            uint32_t w[4];
            stream_words(seed, (uint32_t)i, xuid, xcount, TAG_EXCH, 0, w);
            ok = u53(w) < exp(-d);
        }
        if (ok) {
            t2r[i] = rj;
            t2r[i + 1] = ri;
            r2t[ri] = i + 1;
            r2t[rj] = i;
            ++acc;
        }
    }
    return acc;
}

/* ------------------------------------------------------------------ 5 */
/* Full PT replay of one size.  spins: R * nsites natural layout, in/out.
 * temps[R]; r2t/t2r in/out; counters in/out: *gsweep (global sweep number),
 * *ksample (sampling sweeps done), *xcount (exchanges done).
 * Records (slot, bond, mag) per replica for each measured sweep into the
 * rec_* arrays (capacity max_rec rows of R); returns rows written. */
int64_t or_ising_pt(int L, int dim, int R, int8_t* spins, const double* temps, double J, double h,
                    uint64_t seed, int32_t* r2t, int32_t* t2r, uint64_t* gsweep, uint64_t* ksample,
                    uint64_t* xcount, int64_t* accepted, int64_t warmup, int64_t samples,
                    int exchange_every, int measure_every, int32_t* rec_t, int64_t* rec_b,
                    int64_t* rec_m, int64_t max_rec) {
    int64_t n = nsites(L, dim);
    uint32_t* thr = (uint32_t*)malloc(sizeof(uint32_t) * 16 * (size_t)R);
    double* betas = (double*)malloc(sizeof(double) * (size_t)R);
    double* en = (double*)malloc(sizeof(double) * (size_t)R);
    int64_t* bb = (int64_t*)malloc(sizeof(int64_t) * (size_t)R);
    int64_t* mm = (int64_t*)malloc(sizeof(int64_t) * (size_t)R);
    for (int t = 0; t < R; ++t) {
        betas[t] = 1.0 / temps[t];
        or_ising_thresholds(dim, betas[t], J, h, thr + 16 * t);
    }
    int64_t rows = 0;
    for (int64_t w = 0; w < warmup; ++w) {
        for (int r = 0; r < R; ++r)
            for (int c = 0; c < 2; ++c)
                or_ising_halfsweep(L, dim, spins + (size_t)r * n, c, seed, or_replica_uid(L, r),
                                   *gsweep, thr + 16 * r2t[r]);
        ++*gsweep;
    }
    for (int64_t s = 0; s < samples; ++s) {
        for (int r = 0; r < R; ++r)
            for (int c = 0; c < 2; ++c)
                or_ising_halfsweep(L, dim, spins + (size_t)r * n, c, seed, or_replica_uid(L, r),
                                   *gsweep, thr + 16 * r2t[r]);
        uint64_t k = *ksample;
        int do_m = ((k + 1) % (uint64_t)measure_every) == 0;
        int do_x = ((k + 1) % (uint64_t)exchange_every) == 0;
        if (do_m || do_x) {
            for (int r = 0; r < R; ++r) {
                or_ising_measure(L, dim, spins + (size_t)r * n, &bb[r], &mm[r]);
                double t1 = J * (double)bb[r];
                double t2 = h * (double)mm[r];
                en[r] = -t1 - t2;
            }
        }
        if (do_m && rows < max_rec) {
            for (int r = 0; r < R; ++r) {
                rec_t[rows * R + r] = r2t[r];
                rec_b[rows * R + r] = bb[r];
                rec_m[rows * R + r] = mm[r];
            }
            ++rows;
        }
        if (do_x) {
            *accepted += or_exchange(R, betas, en, r2t, t2r, (int)(*xcount & 1), seed,
                                     or_exchange_uid(L), *xcount);
            ++*xcount;
        }
        ++*ksample;
        ++*gsweep;
    }
    free(thr); free(betas); free(en); free(bb); free(mm);
    return rows;
}

/* ------------------------------------------------------------------ 6 */
typedef struct { uint64_t s[4]; } xo256;

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t splitmix64(uint64_t* st) {
    uint64_t z = (*st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void or_xo_seed(xo256* g, uint64_t seed) {
    uint64_t st = seed;
    for (int i = 0; i < 4; ++i) g->s[i] = splitmix64(&st);
}

static inline uint64_t xo_next(xo256* g) {
    uint64_t* s = g->s;
    uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

/* rand 0.8 UniformInt<u64>::sample_single for [0, range). */
static inline uint64_t xo_range(xo256* g, uint64_t range) {
    int lz = __builtin_clzll(range);
    uint64_t zone = (range << lz) - 1;
    for (;;) {
        uint64_t v = xo_next(g);
        unsigned __int128 p = (unsigned __int128)v * range;
        uint64_t lo = (uint64_t)p, hi = (uint64_t)(p >> 64);
        if (lo <= zone) return hi;
    }
}

static inline double xo_f64(xo256* g) {
    return (double)(xo_next(g) >> 11) * (1.0 / 9007199254740992.0);
}

/* The same generator for the other oracle files. */
uint64_t or_xo_range(xo256* g, uint64_t range) { return xo_range(g, range); }
double or_xo_f64(xo256* g) { return xo_f64(g); }

/* Neighbour table: reference order (-x,+x,-y,+y,-z,+z in lattice.rs terms). */
int32_t* or_ref_neighbours(int L, int dim) {
    int64_t n = nsites(L, dim);
    int z = 2 * dim;
    int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n * z));
    if (dim == 3) {
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j)
                for (int k = 0; k < L; ++k) {
                    int64_t idx = ((int64_t)i * L + j) * L + k;
                    int32_t* p = nb + idx * 6;
                    p[0] = (int32_t)((((i + L - 1) % L) * L + j) * L + k);
                    p[1] = (int32_t)((((i + 1) % L) * L + j) * L + k);
                    p[2] = (int32_t)(((i * L + (j + L - 1) % L) * L) + k);
                    p[3] = (int32_t)(((i * L + (j + 1) % L) * L) + k);
                    p[4] = (int32_t)((i * L + j) * L + (k + L - 1) % L);
                    p[5] = (int32_t)((i * L + j) * L + (k + 1) % L);
                }
    } else {
        for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
                int64_t idx = (int64_t)i * L + j;
                int32_t* p = nb + idx * 4;
                p[0] = (int32_t)(((i + L - 1) % L) * L + j);
                p[1] = (int32_t)(((i + 1) % L) * L + j);
                p[2] = (int32_t)(i * L + (j + L - 1) % L);
                p[3] = (int32_t)(i * L + (j + 1) % L);
            }
    }
    return nb;
}

void or_free(void* p) { free(p); }

void or_ref_randomise(int8_t* spins, int64_t n, xo256* g) {
    for (int64_t i = 0; i < n; ++i) spins[i] = (xo_next(g) < 0x8000000000000000ull) ? 1 : -1;
}

/* src/metropolis.rs:8-27: `attempts` random-site updates (a sweep is n). */
static void ref_attempts(int8_t* spins, int64_t n, int64_t attempts, const int32_t* nb, int z,
                         double beta, double J, double h, xo256* g) {
    for (int64_t a = 0; a < attempts; ++a) {
        int64_t idx = (int64_t)xo_range(g, (uint64_t)n);
        double s = (double)spins[idx];
        double sum = 0.0;
        const int32_t* p = nb + idx * z;
        for (int k = 0; k < z; ++k) sum += (double)spins[p[k]];
        double dE = 2.0 * s * (J * sum + h);
        if (dE < 0.0 || xo_f64(g) < exp(-beta * dE)) spins[idx] = (int8_t)(-spins[idx]);
    }
}

/* src/metropolis.rs:8-27, one random-site sweep of n attempts. */
void or_ref_metropolis_sweep(int8_t* spins, int64_t n, const int32_t* nb, int z, double beta,
                             double J, double h, xo256* g) {
    ref_attempts(spins, n, n, nb, z, beta, J, h, g);
}

/* Random-site Metropolis run with per-sweep (e, |m|) per site recorded. */
void or_ref_run(int L, int dim, double T, double J, double h, uint64_t seed, int64_t warmup,
                int64_t samples, double* e_out, double* m_out) {
    int64_t n = nsites(L, dim);
    int z = 2 * dim;
    int8_t* spins = (int8_t*)malloc((size_t)n);
    int32_t* nb = or_ref_neighbours(L, dim);
    xo256 g;
    or_xo_seed(&g, seed);
    or_ref_randomise(spins, n, &g);
    double beta = 1.0 / T;
    for (int64_t w = 0; w < warmup; ++w) or_ref_metropolis_sweep(spins, n, nb, z, beta, J, h, &g);
    for (int64_t s = 0; s < samples; ++s) {
        or_ref_metropolis_sweep(spins, n, nb, z, beta, J, h, &g);
        int64_t b, m;
        or_ising_measure(L, dim, spins, &b, &m);
        double e = -J * (double)b - h * (double)m;
        e_out[s] = e / (double)n;
        m_out[s] = fabs((double)m) / (double)n;
    }
    free(spins);
    free(nb);
}

/* Timed checkerboard replay (same stream as the GPU), `threads` replicas. */
typedef struct {
    int L, dim;
    uint64_t seed;
    int r;
    int64_t sweeps;
    const uint32_t* thr;
} replay_arg;

static void* replay_worker(void* vp) {
    replay_arg* a = (replay_arg*)vp;
    int64_t n = nsites(a->L, a->dim);
    int8_t* spins = (int8_t*)malloc((size_t)n);
    uint32_t uid = or_replica_uid(a->L, a->r);
    or_ising_hot_start(a->L, a->dim, a->seed, uid, spins);
    for (int64_t s = 0; s < a->sweeps; ++s)
        for (int c = 0; c < 2; ++c)
            or_ising_halfsweep(a->L, a->dim, spins, c, a->seed, uid, (uint64_t)s, a->thr);
    free(spins);
    return NULL;
}

double or_replay_bench(int L, int dim, double T, int64_t sweeps, int threads, uint64_t seed,
                       double* flips) {
    uint32_t thr[16];
    or_ising_thresholds(dim, 1.0 / T, 1.0, 0.0, thr);
    replay_arg* args = (replay_arg*)calloc((size_t)threads, sizeof(replay_arg));
    pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int i = 0; i < threads; ++i) {
        args[i].L = L; args[i].dim = dim; args[i].seed = seed; args[i].r = i;
        args[i].sweeps = sweeps; args[i].thr = thr;
        pthread_create(&tid[i], NULL, replay_worker, &args[i]);
    }
    for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    *flips = (double)nsites(L, dim) * (double)sweeps * (double)threads;
    free(args); free(tid);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------------------ 7 */
/* src/bin/gpu_fss.rs:327-412, deviations from the full-sample value. */
void or_jackknife(const double* e, const double* m, int64_t n, double beta, double n3,
                  int n_blocks, double out[12]) {
    for (int i = 0; i < 12; ++i) out[i] = 0.0;
    if (n < n_blocks || n_blocks < 2) return;
    int64_t bs = n / n_blocks;
    int64_t nu = bs * n_blocks;
    double se = 0, se2 = 0, sm = 0, sm2 = 0, sm4 = 0;
    for (int64_t i = 0; i < nu; ++i) {
        double a = e[i], b = m[i];
        se += a; se2 += a * a; sm += b; sm2 += b * b; sm4 += (b * b) * (b * b);
    }
    double s = (double)nu;
    double ae = se / s, ae2 = se2 / s, am = sm / s, am2 = sm2 / s, am4 = sm4 / s;
    double cv = beta * beta * (ae2 - ae * ae) * n3;
    double chi = beta * (am2 - am * am) * n3;
    double full[6] = {ae, am, am2, am4, cv, chi};
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < n_blocks; ++b) {
        int64_t st = (int64_t)b * bs, en = st + bs;
        double be = 0, be2 = 0, bm = 0, bm2 = 0, bm4 = 0;
        for (int64_t i = 0; i < nu; ++i) {
            if (i >= st && i < en) continue;
            double a = e[i], c = m[i];
            be += a; be2 += a * a; bm += c; bm2 += c * c; bm4 += (c * c) * (c * c);
        }
        double sj = (double)(nu - bs);
        double je = be / sj, je2 = be2 / sj, jm = bm / sj, jm2 = bm2 / sj, jm4 = bm4 / sj;
        double jk[6] = {je, jm, jm2, jm4, beta * beta * (je2 - je * je) * n3,
                        beta * (jm2 - jm * jm) * n3};
        for (int k = 0; k < 6; ++k) acc[k] += (jk[k] - full[k]) * (jk[k] - full[k]);
    }
    double nb = (double)n_blocks;
    for (int k = 0; k < 6; ++k) {
        out[2 * k] = full[k];
        out[2 * k + 1] = sqrt(acc[k] * (nb - 1.0) / nb);
    }
}

/* ------------------------------------------------------------------ 8 */
/* Persistent multi-threaded runner of the reference CPU path (section 6) for
 * the timed baseline: every thread owns one replica of every lattice size of
 * the workload (hot start from its own Xoshiro256++ stream, temperature from
 * the workload grid), and a step runs `sweeps` random-site sweeps of each. */
typedef struct {
    int n_sizes, dim, threads;
    int sizes[16];
    int32_t* nb[16];
    int8_t** spins;   /* [threads * n_sizes] */
    xo256* rng;       /* [threads] */
    double* beta;     /* [threads] */
    double frac;      /* sweeps per step (fractions allowed: attempts = frac * n) */
} refbench;

typedef struct { refbench* b; int t; } rb_arg;

static void* rb_worker(void* vp) {
    rb_arg* a = (rb_arg*)vp;
    refbench* b = a->b;
    for (int s = 0; s < b->n_sizes; ++s) {
        int64_t n = nsites(b->sizes[s], b->dim);
        int64_t att = (int64_t)(b->frac * (double)n);
        if (att < 1) att = 1;
        ref_attempts(b->spins[a->t * b->n_sizes + s], n, att, b->nb[s], 2 * b->dim,
                     b->beta[a->t], 1.0, 0.0, &b->rng[a->t]);
    }
    return NULL;
}

void* or_refbench_create(const int* sizes, int n_sizes, int dim, double tmin, double tmax,
                         int threads, uint64_t seed) {
    refbench* b = (refbench*)calloc(1, sizeof(refbench));
    b->n_sizes = n_sizes; b->dim = dim; b->threads = threads;
    b->spins = (int8_t**)calloc((size_t)(threads * n_sizes), sizeof(int8_t*));
    b->rng = (xo256*)calloc((size_t)threads, sizeof(xo256));
    b->beta = (double*)calloc((size_t)threads, sizeof(double));
    for (int s = 0; s < n_sizes; ++s) {
        b->sizes[s] = sizes[s];
        b->nb[s] = or_ref_neighbours(sizes[s], dim);
    }
    for (int t = 0; t < threads; ++t) {
        or_xo_seed(&b->rng[t], seed + (uint64_t)t * 1000);
        double T = threads > 1 ? tmin + (tmax - tmin) * (double)t / (double)(threads - 1) : tmin;
        b->beta[t] = 1.0 / T;
        for (int s = 0; s < n_sizes; ++s) {
            int64_t n = nsites(sizes[s], dim);
            b->spins[t * n_sizes + s] = (int8_t*)malloc((size_t)n);
            or_ref_randomise(b->spins[t * n_sizes + s], n, &b->rng[t]);
        }
    }
    return b;
}

/* Runs one step of `frac` sweeps of every size on every thread; returns wall
 * seconds and the attempted flips in *flips. */
double or_refbench_step(void* h, double frac, double* flips) {
    refbench* b = (refbench*)h;
    b->frac = frac;
    pthread_t* tid = (pthread_t*)calloc((size_t)b->threads, sizeof(pthread_t));
    rb_arg* args = (rb_arg*)calloc((size_t)b->threads, sizeof(rb_arg));
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < b->threads; ++t) {
        args[t].b = b; args[t].t = t;
        pthread_create(&tid[t], NULL, rb_worker, &args[t]);
    }
    for (int t = 0; t < b->threads; ++t) pthread_join(tid[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    double f = 0;
    for (int s = 0; s < b->n_sizes; ++s) {
        int64_t att = (int64_t)(frac * (double)nsites(b->sizes[s], b->dim));
        f += (double)(att < 1 ? 1 : att);
    }
    *flips = f * (double)b->threads;
    free(tid); free(args);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

void or_refbench_destroy(void* h) {
    refbench* b = (refbench*)h;
    if (!b) return;
    for (int i = 0; i < b->threads * b->n_sizes; ++i) free(b->spins[i]);
    for (int s = 0; s < b->n_sizes; ++s) free(b->nb[s]);
    free(b->spins); free(b->rng); free(b->beta); free(b);
}

/* ------------------------------------------------------------------ 7 */
/* Ising on graphs: replay of isg_graph_* (stream tag GRAPH = 7) and the
 * reference's CPU algorithm on a graph (src/bin/gpu_jfit.rs:172-297). */
#define TAG_GRAPH 0x07u
#define GMAXDEG 12
#define GTAB (2 * (GMAXDEG + 1) * (GMAXDEG + 1))

/* CSR adjacency in edge-list order (both directions) and the greedy proper
 * colouring in node order (smallest class unused by coloured neighbours).
 * rowptr[n+1], adj[2m], colour[n]; returns the number of classes, or -1 for
 * a bad edge list or a degree above 12. */
int or_graph_build(int n, const int32_t* edges, int m, int32_t* rowptr, int32_t* adj,
                   int32_t* colour) {
    for (int v = 0; v <= n; ++v) rowptr[v] = 0;
    for (int e = 0; e < m; ++e) {
        int a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || a >= n || b >= n || a == b) return -1;
        ++rowptr[a + 1];
        ++rowptr[b + 1];
    }
    for (int v = 0; v < n; ++v) {
        if (rowptr[v + 1] > GMAXDEG) return -1;
        rowptr[v + 1] += rowptr[v];
    }
    int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int v = 0; v < n; ++v) fill[v] = rowptr[v];
    for (int e = 0; e < m; ++e) {
        int a = edges[2 * e], b = edges[2 * e + 1];
        adj[fill[a]++] = b;
        adj[fill[b]++] = a;
    }
    free(fill);
    int ncol = 0;
    for (int v = 0; v < n; ++v) colour[v] = -1;
    for (int v = 0; v < n; ++v) {
        uint32_t used = 0;
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
            if (colour[adj[j]] >= 0) used |= 1u << colour[adj[j]];
        int c = 0;
        while ((used >> c) & 1u) ++c;
        colour[v] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    return ncol;
}

/* threshold[(own_down*13 + degree)*13 + n_down] at temperature T. */
void or_graph_thresholds(double T, double J, uint32_t tab[GTAB]) {
    double beta = 1.0 / T;
    for (int i = 0; i < GTAB; ++i) tab[i] = 0;
    for (int od = 0; od < 2; ++od)
        for (int dg = 0; dg <= GMAXDEG; ++dg)
            for (int nd = 0; nd <= dg; ++nd) {
                double dE = 2.0 * J * (od ? -1.0 : 1.0) * (double)(dg - 2 * nd);
                uint32_t th;
                if (dE <= 0.0) {
                    th = 0xFFFFFFFFu;
                } else {
                    double f = floor(exp(-beta * dE) * 4294967296.0);
                    if (f < 1.0) f = 1.0;
                    th = (uint32_t)(f - 1.0);
                }
                tab[(od * (GMAXDEG + 1) + dg) * (GMAXDEG + 1) + nd] = th;
            }
}

/* Hot start: down bit of node v of replica r = top bit of word (v & 3) of
 * Philox(c0 = r, c1 = v >> 2, step 0, colour 0xFE). */
void or_graph_hot_start(int n, int R, uint64_t seed, uint8_t* spins) {
    uint32_t w[4];
    for (int r = 0; r < R; ++r)
        for (int v = 0; v < n; ++v) {
            if ((v & 3) == 0) stream_words(seed, (uint32_t)v >> 2, (uint32_t)r, 0, TAG_GRAPH, 0xFEu, w);
            spins[(size_t)r * n + v] = (uint8_t)(w[v & 3] >> 31);
        }
}

/* One sweep of replica r (down bits sp[n]): colour classes in order, nodes of
 * a class independent of each other. */
void or_graph_sweep(int n, const int32_t* rowptr, const int32_t* adj, const int32_t* colour,
                    int ncol, uint8_t* sp, uint32_t replica, uint64_t seed, uint64_t sweep,
                    const uint32_t* tab) {
    uint32_t w[4];
    for (int c = 0; c < ncol; ++c)
        for (int v = 0; v < n; ++v) {
            if (colour[v] != c) continue;
            int nd = 0;
            for (int j = rowptr[v]; j < rowptr[v + 1]; ++j) nd += sp[adj[j]];
            int d = sp[v];
            int deg = rowptr[v + 1] - rowptr[v];
            uint32_t th = tab[(d * (GMAXDEG + 1) + deg) * (GMAXDEG + 1) + nd];
            stream_words(seed, (uint32_t)v >> 2, replica, sweep, TAG_GRAPH, (uint32_t)c, w);
            if (w[v & 3] <= th) sp[v] = (uint8_t)(d ^ 1);
        }
}

/* Bond sum over edges and magnetisation. */
void or_graph_measure(int n, const int32_t* rowptr, const int32_t* adj, const uint8_t* sp,
                      int64_t* bond, int64_t* mag) {
    int64_t b = 0, m = 0;
    for (int v = 0; v < n; ++v) {
        int s = 1 - 2 * (int)sp[v];
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
            if (adj[j] > v) b += s * (1 - 2 * (int)sp[adj[j]]);
        m += s;
    }
    *bond = b;
    *mag = m;
}

/* Full replay of isg_graph_step (n_warm) followed by isg_graph_pt_run
 * (n_sample, ee, me) with the counters carried in/out as in or_ising_pt. */
int64_t or_graph_pt(int n, const int32_t* edges, int m, int R, uint8_t* spins,
                    const double* temps, double J, uint64_t seed, int32_t* r2t, int32_t* t2r,
                    uint64_t* gsweep, uint64_t* ksample, uint64_t* xcount, int64_t* accepted,
                    int64_t n_warm, int64_t n_sample, int ee, int me, int32_t* rec_t,
                    int64_t* rec_b, int64_t* rec_m, int64_t max_rec) {
    int32_t* rowptr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t* adj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * m > 0 ? 2 * m : 1));
    int32_t* colour = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int ncol = or_graph_build(n, edges, m, rowptr, adj, colour);
    uint32_t* tab = (uint32_t*)malloc(sizeof(uint32_t) * GTAB * (size_t)R);
    double* betas = (double*)malloc(sizeof(double) * (size_t)R);
    double* en = (double*)malloc(sizeof(double) * (size_t)R);
    for (int t = 0; t < R; ++t) {
        or_graph_thresholds(temps[t], J, tab + (size_t)t * GTAB);
        betas[t] = 1.0 / temps[t];
    }
    int64_t rows = 0;
    for (int64_t w = 0; w < n_warm; ++w) {
        for (int r = 0; r < R; ++r)
            or_graph_sweep(n, rowptr, adj, colour, ncol, spins + (size_t)r * n, (uint32_t)r, seed,
                           *gsweep, tab + (size_t)r2t[r] * GTAB);
        ++*gsweep;
    }
    for (int64_t s = 0; s < n_sample; ++s) {
        for (int r = 0; r < R; ++r)
            or_graph_sweep(n, rowptr, adj, colour, ncol, spins + (size_t)r * n, (uint32_t)r, seed,
                           *gsweep, tab + (size_t)r2t[r] * GTAB);
        const int do_m = ((*ksample + 1) % (uint64_t)me) == 0;
        const int do_x = ((*ksample + 1) % (uint64_t)ee) == 0;
        if (do_m || do_x) {
            for (int r = 0; r < R; ++r) {
                int64_t b, mg;
                or_graph_measure(n, rowptr, adj, spins + (size_t)r * n, &b, &mg);
                en[r] = -(J * (double)b);
                if (do_m && rows < max_rec) {
                    rec_t[rows * R + r] = r2t[r];
                    rec_b[rows * R + r] = b;
                    rec_m[rows * R + r] = mg;
                }
            }
            if (do_m) ++rows;
        }
        if (do_x) {
            *accepted += or_exchange(R, betas, en, r2t, t2r, (int)(*xcount & 1), seed,
                                     0xFFFFFFFFu, *xcount);
            ++*xcount;
        }
        ++*ksample;
        ++*gsweep;
    }
    free(rowptr); free(adj); free(colour); free(tab); free(betas); free(en);
    return rows;
}

/* The reference's CPU algorithm on a graph (gpu_jfit.rs:172-262 with
 * metropolis.rs:8-27): R replicas hot-started from Xoshiro256++ seeded
 * seed + 1000 r, one shared Xoshiro256++(seed) for all sweeps and exchanges,
 * random-site Metropolis sweeps of n attempts, E and M every sample,
 * exchange every ee samples.  Writes per-temperature sums
 * out[t*6 + {0..5}] = sum e, sum e^2, sum |m|, sum m^2, sum m^4, count. */
void or_graph_ref_pt(int n, const int32_t* edges, int m, int R, const double* temps, double J,
                     uint64_t seed, int64_t warmup, int64_t samples, int ee, double* out) {
    int32_t* rowptr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t* adj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * m > 0 ? 2 * m : 1));
    int32_t* colour = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    or_graph_build(n, edges, m, rowptr, adj, colour);
    int8_t* sp = (int8_t*)malloc((size_t)n * R);
    int32_t* r2t = (int32_t*)malloc(sizeof(int32_t) * R);
    int32_t* t2r = (int32_t*)malloc(sizeof(int32_t) * R);
    double* betas = (double*)malloc(sizeof(double) * R);
    double* en = (double*)malloc(sizeof(double) * R);
    for (int r = 0; r < R; ++r) {
        xo256 gr;
        or_xo_seed(&gr, seed + (uint64_t)r * 1000u);
        or_ref_randomise(sp + (size_t)r * n, n, &gr);
        r2t[r] = t2r[r] = r;
        betas[r] = 1.0 / temps[r];
    }
    for (int i = 0; i < 6 * R; ++i) out[i] = 0.0;
    xo256 g;
    or_xo_seed(&g, seed);
    const double nn = (double)n;
    for (int64_t s = -warmup; s < samples; ++s) {
        for (int r = 0; r < R; ++r) {
            int8_t* x = sp + (size_t)r * n;
            double beta = betas[r2t[r]];
            for (int a = 0; a < n; ++a) {
                int idx = (int)xo_range(&g, (uint64_t)n);
                double sum = 0.0;
                for (int j = rowptr[idx]; j < rowptr[idx + 1]; ++j) sum += (double)x[adj[j]];
                double dE = 2.0 * (double)x[idx] * (J * sum);
                if (dE < 0.0 || xo_f64(&g) < exp(-beta * dE)) x[idx] = (int8_t)(-x[idx]);
            }
            if (s < 0) continue;
            int64_t b = 0, mg = 0;
            for (int v = 0; v < n; ++v) {
                for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
                    if (adj[j] > v) b += x[v] * x[adj[j]];
                mg += x[v];
            }
            double e = -J * (double)b;
            double e_per = e / nn, m_per = fabs((double)mg / nn);
            en[r] = e;
            double* o = out + (size_t)r2t[r] * 6;
            o[0] += e_per;
            o[1] += e_per * e_per;
            o[2] += m_per;
            o[3] += m_per * m_per;
            o[4] += (m_per * m_per) * (m_per * m_per);
            o[5] += 1.0;
        }
        if (s >= 0 && (s + 1) % ee == 0) {
            /* replica_exchange (parallel_tempering.rs:5-36) drawing from the
             * shared generator */
            for (int i = (int)((s / ee) & 1); i + 1 < R; i += 2) {
                int ri = t2r[i], rj = t2r[i + 1];
                double d = (betas[i] - betas[i + 1]) * (en[rj] - en[ri]);
                if (d < 0.0 || xo_f64(&g) < exp(-d)) {
                    t2r[i] = rj;
                    t2r[i + 1] = ri;
                    r2t[ri] = i + 1;
                    r2t[rj] = i;
                }
            }
        }
    }
    free(rowptr); free(adj); free(colour); free(sp); free(r2t); free(t2r); free(betas); free(en);
}
