// isg_stats.cpp — host statistics of the drop-in driver.
//
// Leave-one-block-out jackknife of an (e, |m|) series, restated from
// jackknife_observables (src/bin/gpu_fss.rs:327-412): block_size = n / n_blocks
// on the first block_size*n_blocks samples, Cv = beta^2 (<e^2> - <e>^2) N,
// chi = beta (<m^2> - <m>^2) N, errors sqrt((nb-1)/nb * sum (jk - full)^2)
// about the full-sample value.  m^4 is formed as (m*m)*(m*m), the rounding of
// Rust's powi(4); the file is compiled with -ffp-contract=off so no product is
// fused into an add, matching Rust's f64 arithmetic bit for bit.
#include <math.h>
#include <stdint.h>

#include <string>

#include "isg.h"

namespace isg {
int fail(int code, const std::string& msg);
}

extern "C" int isg_jackknife(const double* e, const double* m, int64_t n, double beta,
                             double n3, int n_blocks, double* out) {
    if (!out || (n > 0 && (!e || !m))) return isg::fail(ISG_ERR_ARG, "isg_jackknife: NULL argument");
    for (int i = 0; i < 12; ++i) out[i] = 0.0;
    if (n < n_blocks || n_blocks < 2) return ISG_OK;
    const int64_t bs = n / n_blocks;
    const int64_t nu = bs * n_blocks;
    double se = 0.0, se2 = 0.0, sm = 0.0, sm2 = 0.0, sm4 = 0.0;
    for (int64_t i = 0; i < nu; ++i) {
        const double a = e[i], b = m[i];
        se += a;
        se2 += a * a;
        sm += b;
        sm2 += b * b;
        sm4 += (b * b) * (b * b);
    }
    const double s = (double)nu;
    const double ae = se / s, ae2 = se2 / s, am = sm / s, am2 = sm2 / s, am4 = sm4 / s;
    const double cv = beta * beta * (ae2 - ae * ae) * n3;
    const double chi = beta * (am2 - am * am) * n3;
    const double full[6] = {ae, am, am2, am4, cv, chi};
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    // Each leave-one-block-out sum runs over the other samples in sample
    // order, as the reference loop does, so the rounding is the same.
    for (int b = 0; b < n_blocks; ++b) {
        const int64_t st = (int64_t)b * bs, en = st + bs;
        double be = 0.0, be2 = 0.0, bm = 0.0, bm2 = 0.0, bm4 = 0.0;
        for (int64_t i = 0; i < nu; ++i) {
            if (i >= st && i < en) continue;
            const double a = e[i], c = m[i];
            be += a;
            be2 += a * a;
            bm += c;
            bm2 += c * c;
            bm4 += (c * c) * (c * c);
        }
        const double sj = (double)(nu - bs);
        const double je = be / sj, je2 = be2 / sj, jm = bm / sj, jm2 = bm2 / sj, jm4 = bm4 / sj;
        const double jk[6] = {je, jm, jm2, jm4, beta * beta * (je2 - je * je) * n3,
                              beta * (jm2 - jm * jm) * n3};
        for (int k = 0; k < 6; ++k) {
            const double d = jk[k] - full[k];
            acc[k] += d * d;
        }
    }
    const double nb = (double)n_blocks;
    for (int k = 0; k < 6; ++k) {
        out[2 * k] = full[k];
        out[2 * k + 1] = sqrt(acc[k] * (nb - 1.0) / nb);
    }
    return ISG_OK;
}
