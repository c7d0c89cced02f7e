/*
 * cont_oracle.c — CPU ORACLE (FP64) for the continuous-spin O(n) path.
 *
 * TEST INFRASTRUCTURE ONLY (see isg_oracle.c).  Natural layout, n_comp
 * doubles per site interleaved (src/cuda/continuous_spin_kernel.cu:6).
 *
 *  - hot start: the device's ISG_TAG_CINIT formula (z, phi uniform for O(3) as
 *    src/cuda/gpu_lattice_continuous.rs:49-56; uniform angle for O(2) as
 *    src/xy/mod.rs:42-45) evaluated in FP64;
 *  - overrelaxation: S' = 2 (S.h)/|h|^2 h - S (src/heisenberg/overrelax.rs:16-49,
 *    src/cuda/continuous_spin_kernel.cu:88-142), one colour at a time;
 *  - Metropolis: the cone proposal of src/heisenberg/metropolis.rs:54-92 with
 *    cos(theta) = 1 - u0 (1 - cos delta), phi = 2 pi u1, and the same
 *    perpendicular frame; O(2) rotates by delta (2 u0 - 1); accept if dE <= 0
 *    or u2 < exp(-beta dE) (src/heisenberg/metropolis.rs:26-35), with u0..u2
 *    the 24-bit uniforms of the ISG_TAG_CMETRO Philox words (O(2): the block of
 *    colour index c >> 1, words 0 and 2 for even c, 1 and 3 for odd c);
 *  - measure: E = -J sum_bonds S.S' and M (src/heisenberg/mod.rs:59-74,
 *    src/xy/mod.rs:50-64) plus the helicity bond sums.
 * The GPU computes in FP32, so agreement is within FP32 rounding, and an
 * acceptance decision can differ where u2 is within rounding of exp(-beta dE).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#define TAG_CINIT 0x04u
#define TAG_CMETRO 0x05u

static void words(uint64_t seed, uint32_t uid, uint32_t index, uint64_t step, uint32_t tag,
                  uint32_t colour, uint32_t out[4]) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {uid, index, (uint32_t)step,
                       (tag << 24) | (colour << 16) | ((uint32_t)(step >> 32) & 0xFFFFu)};
    or_philox4x32_10(ctr, key, out);
}

static double u24(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }

static const double PI = 3.14159265358979323846;

void or_cont_hot_start(int L, int nc, uint64_t seed, uint32_t uid, double* s) {
    int64_t n = (int64_t)L * L * L;
    for (int64_t i = 0; i < n; ++i) {
        uint32_t w[4];
        words(seed, uid, (uint32_t)i, 0, TAG_CINIT, 0, w);
        if (nc == 3) {
            double z = 2.0 * u24(w[0]) - 1.0;
            double ph = 2.0 * PI * u24(w[1]);
            double r = sqrt(fmax(0.0, 1.0 - z * z));
            s[i * 3 + 0] = r * cos(ph);
            s[i * 3 + 1] = r * sin(ph);
            s[i * 3 + 2] = z;
        } else {
            double ph = 2.0 * PI * u24(w[0]);
            s[i * 2 + 0] = cos(ph);
            s[i * 2 + 1] = sin(ph);
        }
    }
}

static int64_t idx3(int L, int x, int y, int z) { return ((int64_t)z * L + y) * L + x; }

static void field(int L, int nc, const double* s, int x, int y, int z, double h[3]) {
    int xs[6] = {(x + 1) % L, (x + L - 1) % L, x, x, x, x};
    int ys[6] = {y, y, (y + 1) % L, (y + L - 1) % L, y, y};
    int zs[6] = {z, z, z, z, (z + 1) % L, (z + L - 1) % L};
    h[0] = h[1] = h[2] = 0.0;
    for (int d = 0; d < 6; ++d) {
        const double* p = s + idx3(L, xs[d], ys[d], zs[d]) * nc;
        for (int k = 0; k < nc; ++k) h[k] += p[k];
    }
}

void or_cont_overrelax(int L, int nc, double* s, int colour, double J) {
    (void)J;
    for (int z = 0; z < L; ++z)
        for (int y = 0; y < L; ++y)
            for (int x = 0; x < L; ++x) {
                if (((x + y + z) & 1) != colour) continue;
                double h[3];
                field(L, nc, s, x, y, z, h);
                double h2 = 0, sh = 0;
                double* v = s + idx3(L, x, y, z) * nc;
                for (int k = 0; k < nc; ++k) {
                    h2 += h[k] * h[k];
                    sh += v[k] * h[k];
                }
                if (h2 < 1e-20) continue;
                double sc = 2.0 * sh / h2;
                for (int k = 0; k < nc; ++k) v[k] = sc * h[k] - v[k];
            }
}

void or_cont_metropolis(int L, int nc, double* s, int colour, uint64_t seed, uint32_t uid,
                        uint64_t sweep, double beta, double J, double delta, int64_t* accepted) {
    double cd = cos(delta < PI ? delta : PI);
    int64_t acc = 0;
    for (int z = 0; z < L; ++z)
        for (int y = 0; y < L; ++y)
            for (int x = 0; x < L; ++x) {
                if (((x + y + z) & 1) != colour) continue;
                int64_t i = idx3(L, x, y, z);
                double h[3];
                field(L, nc, s, x, y, z, h);
                double* v = s + i * nc;
                uint32_t w[4];
                const uint32_t ci = (uint32_t)(i >> 1);  /* colour index */
                /* O(3): one block per site; O(2): one block per pair of colour
                   indices (2j, 2j+1), words 0 and 2 for the even, 1 and 3 for the odd */
                words(seed, uid, nc == 3 ? ci : ci >> 1, sweep, TAG_CMETRO, (uint32_t)colour, w);
                if (nc == 2 && (ci & 1u)) {
                    w[0] = w[1];
                    w[2] = w[3];
                }
                double nv[3];
                if (nc == 3) {
                    double ct = 1.0 - u24(w[0]) * (1.0 - cd);
                    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
                    double ph = 2.0 * PI * u24(w[1]);
                    double tx = fabs(v[0]) < 0.9 ? 1.0 : 0.0, ty = 1.0 - tx;
                    double ts = tx * v[0] + ty * v[1];
                    double ux = tx - ts * v[0], uy = ty - ts * v[1], uz = -ts * v[2];
                    double un = sqrt(ux * ux + uy * uy + uz * uz);
                    ux /= un; uy /= un; uz /= un;
                    double vx = v[1] * uz - v[2] * uy, vy = v[2] * ux - v[0] * uz,
                           vz = v[0] * uy - v[1] * ux;
                    double a = st * cos(ph), b = st * sin(ph);
                    nv[0] = a * ux + b * vx + ct * v[0];
                    nv[1] = a * uy + b * vy + ct * v[1];
                    nv[2] = a * uz + b * vz + ct * v[2];
                    double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
                    for (int k = 0; k < 3; ++k) nv[k] /= nn;
                } else {
                    double an = delta * (2.0 * u24(w[0]) - 1.0);
                    double c = cos(an), sn = sin(an);
                    nv[0] = v[0] * c - v[1] * sn;
                    nv[1] = v[1] * c + v[0] * sn;
                }
                double dot = 0;
                for (int k = 0; k < nc; ++k) dot += (nv[k] - v[k]) * h[k];
                double dE = -J * dot;
                if (dE <= 0.0 || u24(w[2]) < exp(-beta * dE)) {
                    for (int k = 0; k < nc; ++k) v[k] = nv[k];
                    ++acc;
                }
            }
    if (accepted) *accepted += acc;
}

/* out[10] = E, Mx, My, Mz, C_x, C_y, C_z, S_x, S_y, S_z */
void or_cont_measure(int L, int nc, const double* s, double out[10]) {
    for (int q = 0; q < 10; ++q) out[q] = 0.0;
    for (int z = 0; z < L; ++z)
        for (int y = 0; y < L; ++y)
            for (int x = 0; x < L; ++x) {
                const double* a = s + idx3(L, x, y, z) * nc;
                for (int k = 0; k < nc; ++k) out[1 + k] += a[k];
                const double* f[3] = {s + idx3(L, (x + 1) % L, y, z) * nc,
                                      s + idx3(L, x, (y + 1) % L, z) * nc,
                                      s + idx3(L, x, y, (z + 1) % L) * nc};
                for (int ax = 0; ax < 3; ++ax) {
                    double d = 0;
                    for (int k = 0; k < nc; ++k) d += a[k] * f[ax][k];
                    out[0] -= d;
                    out[4 + ax] += d;
                    out[7 + ax] += a[0] * f[ax][1] - a[1] * f[ax][0];
                }
            }
}

/* Reference CPU Heisenberg path (src/heisenberg/metropolis.rs:10-37 random-site
 * sweep with the cone proposal, then src/heisenberg/overrelax.rs:16-49 sequential
 * OR, combined as src/heisenberg/sweep.rs:50-62), driven by Philox words. */
void or_cont_ref_sweep(int L, double* s, double beta, double J, double delta, uint64_t seed,
                       uint64_t sweep, int n_or) {
    int64_t n = (int64_t)L * L * L;
    double cd = cos(delta);
    for (int64_t a = 0; a < n; ++a) {
        uint32_t w[4];
        words(seed, 0xFFFFFFFEu, (uint32_t)a, sweep, TAG_CMETRO, 0, w);
        int64_t i = (int64_t)(((uint64_t)w[3] * (uint64_t)n) >> 32);
        int x = (int)(i % L), y = (int)((i / L) % L), z = (int)(i / ((int64_t)L * L));
        double h[3];
        field(L, 3, s, x, y, z, h);
        double* v = s + i * 3;
        double ct = 1.0 - u24(w[0]) * (1.0 - cd);
        double st = sqrt(fmax(0.0, 1.0 - ct * ct));
        double ph = 2.0 * PI * u24(w[1]);
        double tx = fabs(v[0]) < 0.9 ? 1.0 : 0.0, ty = 1.0 - tx;
        double ts = tx * v[0] + ty * v[1];
        double ux = tx - ts * v[0], uy = ty - ts * v[1], uz = -ts * v[2];
        double un = sqrt(ux * ux + uy * uy + uz * uz);
        ux /= un; uy /= un; uz /= un;
        double vx = v[1] * uz - v[2] * uy, vy = v[2] * ux - v[0] * uz, vz = v[0] * uy - v[1] * ux;
        double ca = st * cos(ph), sb = st * sin(ph);
        double nv[3] = {ca * ux + sb * vx + ct * v[0], ca * uy + sb * vy + ct * v[1],
                        ca * uz + sb * vz + ct * v[2]};
        double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        double dot = 0;
        for (int k = 0; k < 3; ++k) {
            nv[k] /= nn;
            dot += (nv[k] - v[k]) * h[k];
        }
        double dE = -J * dot;
        if (dE < 0.0 || u24(w[2]) < exp(-beta * dE))
            for (int k = 0; k < 3; ++k) v[k] = nv[k];
    }
    for (int r = 0; r < n_or; ++r)
        for (int64_t i = 0; i < n; ++i) {
            int x = (int)(i % L), y = (int)((i / L) % L), z = (int)(i / ((int64_t)L * L));
            double h[3];
            field(L, 3, s, x, y, z, h);
            double h2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
            if (h2 < 1e-30) continue;
            double* v = s + i * 3;
            double sc = 2.0 * (v[0] * h[0] + v[1] * h[1] + v[2] * h[2]) / h2;
            double nv[3] = {sc * h[0] - v[0], sc * h[1] - v[1], sc * h[2] - v[2]};
            double nn = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
            for (int k = 0; k < 3; ++k) v[k] = nv[k] / nn;
        }
}
