/*
 * cgraph_oracle.c — CPU ORACLE (FP64) for continuous spins on graphs.
 *
 * TEST INFRASTRUCTURE ONLY (see isg_oracle.c).  Spins in natural layout,
 * n_comp doubles per node.
 *
 *  1. Replay of the device engine isg_cgraph_* (include/isg.h, ISG_TAG_CGRAPH):
 *     the hot start, one O(3) cone-Metropolis sweep by colour class
 *     (proposal of src/heisenberg/metropolis.rs:54-92 with cos(theta) =
 *     1 - u0 (1 - cos delta), phi = 2 pi u1, accept dE <= 0 or
 *     u2 < exp(-beta dE), metropolis.rs:26-35), one O(2) single-cluster Wolff
 *     flip (src/xy/wolff.rs:15-78) grown depth-first with the device's
 *     per-bond words, and E = -J sum_bonds S.S', M = sum S
 *     (src/heisenberg/mod.rs:56-74, src/xy/mod.rs:47-64).  The device computes
 *     in FP32, so agreement is within FP32 rounding; every sweep reports the
 *     smallest margin of its decisions (|u - p| of an acceptance or bond test,
 *     |p_i p_j| of a sign test), below which the device may decide otherwise.
 *  2. The reference algorithms of run_heisenberg_jfit / run_xy_jfit
 *     (src/bin/gpu_jfit.rs:298-524): hot starts from one shared Xoshiro256++
 *     (random_unit_vector, Marsaglia 1972, heisenberg/mod.rs:41-54;
 *     random_unit_circle, xy/mod.rs:40-45), random-site cone Metropolis sweeps
 *     with delta as given, sequential Wolff flips, E and |M| per sample, the
 *     exchange pass of src/parallel_tempering.rs:5-36 every exchange_every
 *     samples — all drawing from that generator.  Uniform floats in [a, b)
 *     are a + (b - a) u with u = gen::<f64>; statistical oracle only.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
typedef struct { uint64_t s[4]; } xo256;
void or_xo_seed(xo256* g, uint64_t seed);
uint64_t or_xo_range(xo256* g, uint64_t range);
double or_xo_f64(xo256* g);

#define TAG_CGRAPH 0x08u
#define CG_MAXDEG 64
#define TWO_PI 6.283185307179586476925286766559

static void cg_words(uint64_t seed, uint32_t c0, uint32_t c1, uint64_t step, uint32_t field,
                     uint32_t out[4]) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {c0, c1, (uint32_t)step,
                       (TAG_CGRAPH << 24) | (field << 16) | ((uint32_t)(step >> 32) & 0xFFFFu)};
    or_philox4x32_10(ctr, key, out);
}

static double cg_u24(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }

/* CSR (both directions, edge-list order) and greedy colouring in node order;
 * degree at most 64.  Returns the class count or -1. */
int or_cgraph_build(int n, const int32_t* edges, int m, int32_t* rowptr, int32_t* adj,
                    int32_t* colour) {
    for (int v = 0; v <= n; ++v) rowptr[v] = 0;
    for (int e = 0; e < m; ++e) {
        int a = edges[2 * e], b = edges[2 * e + 1];
        if (a < 0 || b < 0 || a >= n || b >= n || a == b) return -1;
        ++rowptr[a + 1];
        ++rowptr[b + 1];
    }
    for (int v = 0; v < n; ++v) {
        if (rowptr[v + 1] > CG_MAXDEG) return -1;
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
    char used[CG_MAXDEG + 2];
    for (int v = 0; v < n; ++v) colour[v] = -1;
    for (int v = 0; v < n; ++v) {
        memset(used, 0, sizeof used);
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
            if (colour[adj[j]] >= 0) used[colour[adj[j]]] = 1;
        int c = 0;
        while (used[c]) ++c;
        colour[v] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    return ncol;
}

/* sp[(r*n + v)*nc + k] */
void or_cgraph_hot_start(int n, int R, int nc, uint64_t seed, double* sp) {
    uint32_t w[4];
    for (int r = 0; r < R; ++r)
        for (int v = 0; v < n; ++v) {
            cg_words(seed, (uint32_t)r, (uint32_t)v, 0, 0xFEu, w);
            double* s = sp + ((size_t)r * n + v) * nc;
            if (nc == 3) {
                double z = 2.0 * cg_u24(w[0]) - 1.0, ph = TWO_PI * cg_u24(w[1]);
                double rr = sqrt(fmax(0.0, 1.0 - z * z));
                s[0] = rr * cos(ph);
                s[1] = rr * sin(ph);
                s[2] = z;
            } else {
                double ph = TWO_PI * cg_u24(w[0]);
                s[0] = cos(ph);
                s[1] = sin(ph);
            }
        }
}

/* Cone proposal around s (heisenberg/metropolis.rs:54-92) from ct = cos(theta)
 * and phi. */
static void cone(const double* s, double ct, double ph, double* w) {
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double tx = fabs(s[0]) < 0.9 ? 1.0 : 0.0, ty = 1.0 - tx;
    double ts = tx * s[0] + ty * s[1];
    double ux = tx - ts * s[0], uy = ty - ts * s[1], uz = -ts * s[2];
    double un = sqrt(ux * ux + uy * uy + uz * uz);
    ux /= un;
    uy /= un;
    uz /= un;
    double vx = s[1] * uz - s[2] * uy, vy = s[2] * ux - s[0] * uz, vz = s[0] * uy - s[1] * ux;
    double a = st * cos(ph), b = st * sin(ph);
    w[0] = a * ux + b * vx + ct * s[0];
    w[1] = a * uy + b * vy + ct * s[1];
    w[2] = a * uz + b * vz + ct * s[2];
    double wn = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    w[0] /= wn;
    w[1] /= wn;
    w[2] /= wn;
}

/* One O(3) sweep of the device engine on replica `replica` (sp = n*3 doubles).
 * Returns the accepted count; *margin = min over uphill proposals of
 * |u2 - exp(-beta dE)|. */
int64_t or_cgraph_metro_sweep(int n, const int32_t* rowptr, const int32_t* adj,
                              const int32_t* colour, int ncol, double* sp, uint32_t replica,
                              uint64_t seed, uint64_t sweep, double beta, double J,
                              double cos_delta, double* margin) {
    int64_t acc = 0;
    uint32_t w4[4];
    for (int c = 0; c < ncol; ++c)
        for (int v = 0; v < n; ++v) {
            if (colour[v] != c) continue;
            double h[3] = {0.0, 0.0, 0.0};
            for (int j = rowptr[v]; j < rowptr[v + 1]; ++j)
                for (int k = 0; k < 3; ++k) h[k] += sp[(size_t)adj[j] * 3 + k];
            double* s = sp + (size_t)v * 3;
            cg_words(seed, replica, (uint32_t)v, sweep, (uint32_t)c, w4);
            double w[3];
            cone(s, 1.0 - cg_u24(w4[0]) * (1.0 - cos_delta), TWO_PI * cg_u24(w4[1]), w);
            double dot = 0.0;
            for (int k = 0; k < 3; ++k) dot += (w[k] - s[k]) * h[k];
            double dE = -J * dot;
            int ok = dE <= 0.0;
            if (!ok) {
                double p = exp(-beta * dE), u = cg_u24(w4[2]);
                if (fabs(u - p) < *margin) *margin = fabs(u - p);
                ok = u < p;
            }
            if (ok) {
                for (int k = 0; k < 3; ++k) s[k] = w[k];
                ++acc;
            }
        }
    return acc;
}

/* One O(2) single-cluster flip of the device engine (sp = n*2 doubles).
 * Returns the cluster size; *margin as above. */
int or_cgraph_wolff_sweep(int n, const int32_t* rowptr, const int32_t* adj, double* sp,
                          uint32_t replica, uint64_t seed, uint64_t sweep, double beta, double J,
                          double* margin) {
    uint32_t w[4];
    cg_words(seed, replica, 0xFFFFFFFFu, sweep, 0xFDu, w);
    double ph = TWO_PI * cg_u24(w[0]);
    double rx = cos(ph), ry = sin(ph);
    int start = (int)(((uint64_t)w[1] * (uint64_t)n) >> 32);
    char* in = (char*)calloc((size_t)n, 1);
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* members = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int top = 0, count = 0;
    in[start] = 1;
    stack[top++] = start;
    members[count++] = start;
    while (top > 0) {
        int i = stack[--top];
        double pi = sp[2 * i] * rx + sp[2 * i + 1] * ry;
        for (int k = 0; k < rowptr[i + 1] - rowptr[i]; ++k) {
            if ((k & 3) == 0) cg_words(seed, replica, (uint32_t)i, sweep, 0xC0u + (uint32_t)(k >> 2), w);
            int j = adj[rowptr[i] + k];
            if (in[j]) continue;
            double pj = sp[2 * j] * rx + sp[2 * j + 1] * ry;
            double pp = pi * pj;
            if (fabs(pp) < *margin) *margin = fabs(pp);
            if (pp <= 0.0) continue;
            double p = 1.0 - exp(-2.0 * beta * J * fabs(pi) * fabs(pj));
            double u = cg_u24(w[k & 3]);
            if (fabs(u - p) < *margin) *margin = fabs(u - p);
            if (u < p) {
                in[j] = 1;
                stack[top++] = j;
                members[count++] = j;
            }
        }
    }
    for (int q = 0; q < count; ++q) {
        double* s = sp + 2 * (size_t)members[q];
        double d = s[0] * rx + s[1] * ry;
        s[0] -= 2.0 * d * rx;
        s[1] -= 2.0 * d * ry;
        double nr = sqrt(s[0] * s[0] + s[1] * s[1]);
        s[0] /= nr;
        s[1] /= nr;
    }
    free(in);
    free(stack);
    free(members);
    return count;
}

void or_cgraph_measure(int n, const int32_t* rowptr, const int32_t* adj, const double* sp,
                       int nc, double J, double* e, double* m) {
    double ee = 0.0;
    for (int k = 0; k < nc; ++k) m[k] = 0.0;
    for (int v = 0; v < n; ++v) {
        for (int k = 0; k < nc; ++k) m[k] += sp[(size_t)v * nc + k];
        for (int j = rowptr[v]; j < rowptr[v + 1]; ++j) {
            int u = adj[j];
            if (u <= v) continue;
            double d = 0.0;
            for (int k = 0; k < nc; ++k) d += sp[(size_t)v * nc + k] * sp[(size_t)u * nc + k];
            ee -= J * d;
        }
    }
    *e = ee;
}

/* ------------------------------------------------------------------ 2 */

static void ref_unit_vector(xo256* g, double* s) {
    for (;;) {
        double x = -1.0 + 2.0 * or_xo_f64(g), y = -1.0 + 2.0 * or_xo_f64(g);
        double r2 = x * x + y * y;
        if (r2 >= 1.0) continue;
        double f = 2.0 * sqrt(1.0 - r2);
        s[0] = f * x;
        s[1] = f * y;
        s[2] = 1.0 - 2.0 * r2;
        return;
    }
}

static void ref_heisenberg_sweep(int n, const int32_t* rowptr, const int32_t* adj, double* sp,
                                 double beta, double J, double cos_delta, xo256* g) {
    for (int a = 0; a < n; ++a) {
        int idx = (int)or_xo_range(g, (uint64_t)n);
        double h[3] = {0.0, 0.0, 0.0};
        for (int j = rowptr[idx]; j < rowptr[idx + 1]; ++j)
            for (int k = 0; k < 3; ++k) h[k] += sp[(size_t)adj[j] * 3 + k];
        double* s = sp + (size_t)idx * 3;
        double e_old = -J * (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
        double ct = cos_delta + (1.0 - cos_delta) * or_xo_f64(g);
        double ph = TWO_PI * or_xo_f64(g);
        double w[3];
        cone(s, ct, ph, w);
        double e_new = -J * (w[0] * h[0] + w[1] * h[1] + w[2] * h[2]);
        double dE = e_new - e_old;
        if (dE < 0.0 || or_xo_f64(g) < exp(-beta * dE)) {
            s[0] = w[0];
            s[1] = w[1];
            s[2] = w[2];
        }
    }
}

static void ref_xy_wolff(int n, const int32_t* rowptr, const int32_t* adj, double* sp,
                         double beta, double J, xo256* g, char* in, int32_t* stack) {
    double ph = TWO_PI * or_xo_f64(g);
    double rx = cos(ph), ry = sin(ph);
    int start = (int)or_xo_range(g, (uint64_t)n);
    memset(in, 0, (size_t)n);
    int top = 0;
    in[start] = 1;
    stack[top++] = start;
    while (top > 0) {
        int i = stack[--top];
        double pi = sp[2 * i] * rx + sp[2 * i + 1] * ry;
        for (int j0 = rowptr[i]; j0 < rowptr[i + 1]; ++j0) {
            int j = adj[j0];
            if (in[j]) continue;
            double pj = sp[2 * j] * rx + sp[2 * j + 1] * ry;
            if (pi * pj <= 0.0) continue;
            double p = 1.0 - exp(-2.0 * beta * J * fabs(pi) * fabs(pj));
            if (or_xo_f64(g) < p) {
                in[j] = 1;
                stack[top++] = j;
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        if (!in[i]) continue;
        double* s = sp + 2 * (size_t)i;
        double d = s[0] * rx + s[1] * ry;
        s[0] -= 2.0 * d * rx;
        s[1] -= 2.0 * d * ry;
        double nr = sqrt(s[0] * s[0] + s[1] * s[1]);
        s[0] /= nr;
        s[1] /= nr;
    }
}

/* out[t*6 + {0..5}] = sum e, sum e^2, sum |m|, sum m^2, sum m^4, count per
 * temperature slot (per-node e and |m|). */
void or_cgraph_ref_pt(int n, const int32_t* edges, int m, int R, int nc, const double* temps,
                      double J, uint64_t seed, int64_t warmup, int64_t samples, int ee,
                      double delta, double* out) {
    int32_t* rowptr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t* adj = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * m > 0 ? 2 * m : 1));
    int32_t* colour = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    or_cgraph_build(n, edges, m, rowptr, adj, colour);
    double* sp = (double*)malloc(sizeof(double) * (size_t)n * nc * R);
    int32_t* r2t = (int32_t*)malloc(sizeof(int32_t) * R);
    int32_t* t2r = (int32_t*)malloc(sizeof(int32_t) * R);
    double* en = (double*)malloc(sizeof(double) * R);
    char* in = (char*)malloc((size_t)n);
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    xo256 g;
    or_xo_seed(&g, seed);
    for (int r = 0; r < R; ++r) {
        double* x = sp + (size_t)r * n * nc;
        for (int v = 0; v < n; ++v) {
            if (nc == 3) {
                ref_unit_vector(&g, x + (size_t)v * 3);
            } else {
                double ph = TWO_PI * or_xo_f64(&g);
                x[2 * v] = cos(ph);
                x[2 * v + 1] = sin(ph);
            }
        }
        r2t[r] = t2r[r] = r;
    }
    for (int i = 0; i < 6 * R; ++i) out[i] = 0.0;
    const double cd = cos(delta), nn = (double)n;
    for (int64_t s = -warmup; s < samples; ++s) {
        for (int r = 0; r < R; ++r) {
            double* x = sp + (size_t)r * n * nc;
            double beta = 1.0 / temps[r2t[r]];
            if (nc == 3)
                ref_heisenberg_sweep(n, rowptr, adj, x, beta, J, cd, &g);
            else
                ref_xy_wolff(n, rowptr, adj, x, beta, J, &g, in, stack);
            if (s < 0) continue;
            double e, mv[3];
            or_cgraph_measure(n, rowptr, adj, x, nc, J, &e, mv);
            double m2 = 0.0;
            for (int k = 0; k < nc; ++k) m2 += mv[k] * mv[k];
            double e_per = e / nn, m_abs = sqrt(m2) / nn;
            en[r] = e;
            double* o = out + (size_t)r2t[r] * 6;
            o[0] += e_per;
            o[1] += e_per * e_per;
            o[2] += m_abs;
            o[3] += m_abs * m_abs;
            o[4] += (m_abs * m_abs) * (m_abs * m_abs);
            o[5] += 1.0;
        }
        if (s >= 0 && (s + 1) % ee == 0) {
            for (int i = (int)((s / ee) & 1); i + 1 < R; i += 2) {
                int ri = t2r[i], rj = t2r[i + 1];
                double d = (1.0 / temps[i] - 1.0 / temps[i + 1]) * (en[rj] - en[ri]);
                if (d < 0.0 || or_xo_f64(&g) < exp(-d)) {
                    t2r[i] = rj;
                    t2r[i + 1] = ri;
                    r2t[ri] = i + 1;
                    r2t[rj] = i;
                }
            }
        }
    }
    free(rowptr); free(adj); free(colour); free(sp); free(r2t); free(t2r); free(en);
    free(in); free(stack);
}
