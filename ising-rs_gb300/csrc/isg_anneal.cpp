// isg_anneal.cpp — the annealing finite-size-scaling schedule (`fss --gpu`)
// on the batched Ising engine.
//
// Reference path being replaced (faulknco/ising-rs):
//   src/cuda/fss_gpu.rs:7-39         run_fss_gpu: per size, one LatticeGpu
//                                    swept from t_max down to t_min
//   src/cuda/lattice_gpu.rs:184-251  warm_up / measure: `samples` sweeps, each
//                                    followed by a full spin copy to the host
//                                    and a host E/M sum (energy_magnetisation_host,
//                                    lattice_gpu.rs:285-306)
//
// Here every size is one replica of a single batch and each temperature's
// warm-up and sampling sweeps are isg_ising_run_schedule calls: small lattices
// run them in one launch (one thread-block cluster per lattice), and E/M come
// from integer sums fused into the sweep (no spin copies).  The
// per-temperature statistics follow lattice_gpu.rs:205-251 operation for
// operation in FP64 (host code compiled with -ffp-contract=off):
//   e = E/N, m = |M|/N, m_s = M/N; running sums of e, e^2, m, m^2,
//   ((m*m)*m)*m, m_s, m_s^2 in sample order; averages by division;
//   Cv = ((beta*beta)*(<e^2> - <e>*<e>))*N, chi = (beta*(<m_s^2> - <m_s>*<m_s>))*N
//   with beta = 1/T.
// E = -J*bond - h*M from the exact integer sums (the reference's per-site
// FP64 sum of -J*s*nb/2 - h*s is exact, and equal, for integer and
// half-integer J and h).
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "isg.h"

namespace isg {
int fail(int code, const std::string& msg);
}

namespace {

struct Sums {
    double e = 0, e2 = 0, m = 0, m2 = 0, m4 = 0, ms = 0, ms2 = 0;
};

int anneal_group(const std::vector<int>& sizes, int dim, double t_min, double t_max, int t_steps,
                 double J, double hfield, int64_t warmup, int64_t samples, uint64_t seed,
                 std::vector<std::vector<double>>& obs) {
    const int ns = (int)sizes.size();
    isg_ising* h = nullptr;
    int rc = isg_ising_create(&h, sizes.data(), ns, 1, dim, seed);
    if (rc) return isg::fail(rc, std::string("isg_ising_create: ") + isg_last_error());
    std::vector<double> temps(ns);
    const int64_t chunk = std::min<int64_t>(samples, (int64_t)1 << 16);
    std::vector<int64_t> rb((size_t)chunk * ns), rm((size_t)chunk * ns);
    std::vector<double> nsites(ns);
    for (int s = 0; s < ns; ++s)
        nsites[s] = dim == 3 ? (double)sizes[s] * sizes[s] * sizes[s] : (double)sizes[s] * sizes[s];
    std::vector<Sums> acc(ns);
    for (int step = t_steps - 1; step >= 0 && rc == 0; --step) {
        const double t = t_min + (t_max - t_min) * (double)step / (double)(t_steps - 1);
        std::fill(temps.begin(), temps.end(), t);
        if ((rc = isg_ising_set_temperatures(h, temps.data(), J, hfield))) break;
        if (warmup > 0 &&
            (rc = isg_ising_run_schedule(h, nullptr, warmup, 0, 0, nullptr, nullptr, 0, nullptr)))
            break;
        std::fill(acc.begin(), acc.end(), Sums{});
        for (int64_t done = 0; done < samples && rc == 0;) {
            const int64_t n = std::min<int64_t>(chunk, samples - done);
            int64_t got = 0;
            if ((rc = isg_ising_run_schedule(h, nullptr, n, 1, 0, rb.data(), rm.data(), chunk,
                                             &got)))
                break;
            if (got != n) {
                rc = isg::fail(ISG_ERR_STATE, "isg_fss_anneal: short record set");
                break;
            }
            for (int s = 0; s < ns; ++s) {
                const double n3 = nsites[s];
                Sums& a = acc[s];
                for (int64_t k = 0; k < n; ++k) {
                    const size_t o = (size_t)k * ns + s;
                    const double E = -J * (double)rb[o] - hfield * (double)rm[o];
                    const double M = (double)rm[o];
                    const double e_per = E / n3;
                    const double m_per = std::fabs(M / n3);
                    const double m_signed = M / n3;
                    a.e += e_per;
                    a.e2 += e_per * e_per;
                    a.m += m_per;
                    a.m2 += m_per * m_per;
                    a.m4 += m_per * m_per * m_per * m_per;
                    a.ms += m_signed;
                    a.ms2 += m_signed * m_signed;
                }
            }
            done += n;
        }
        if (rc) break;
        const double beta = 1.0 / t;
        const double sm = (double)samples;
        for (int s = 0; s < ns; ++s) {
            const double n3 = nsites[s];
            const Sums& a = acc[s];
            const double avg_e = a.e / sm, avg_e2 = a.e2 / sm, avg_m = a.m / sm;
            const double avg_m2 = a.m2 / sm, avg_m4 = a.m4 / sm;
            const double avg_ms = a.ms / sm, avg_ms2 = a.ms2 / sm;
            double* row = &obs[s][(size_t)step * 7];
            row[0] = t;
            row[1] = avg_e;
            row[2] = avg_m;
            row[3] = avg_m2;
            row[4] = avg_m4;
            row[5] = beta * beta * (avg_e2 - avg_e * avg_e) * n3;
            row[6] = beta * (avg_ms2 - avg_ms * avg_ms) * n3;
        }
    }
    const int rd = isg_ising_destroy(h);
    return rc ? rc : rd;
}

}  // namespace

extern "C" int isg_fss_anneal(const int* sizes, int n_sizes, int dim, double t_min, double t_max,
                              int t_steps, double J, double hfield, int64_t warmup,
                              int64_t samples, uint64_t seed, double* out) {
    using isg::fail;
    if (!sizes || !out || n_sizes < 1) return fail(ISG_ERR_ARG, "isg_fss_anneal: no sizes");
    if (dim != 2 && dim != 3) return fail(ISG_ERR_ARG, "isg_fss_anneal: dim must be 2 or 3");
    if (t_steps < 2) return fail(ISG_ERR_ARG, "isg_fss_anneal: t_steps must be at least 2");
    if (!(t_min > 0.0) || !(t_max > t_min))
        return fail(ISG_ERR_ARG, "isg_fss_anneal: need 0 < t_min < t_max");
    if (samples < 1 || warmup < 0)
        return fail(ISG_ERR_ARG, "isg_fss_anneal: need samples >= 1 and warmup >= 0");
    if ((int64_t)t_steps * samples > ((int64_t)1 << 40))
        return fail(ISG_ERR_ARG, "isg_fss_anneal: t_steps * samples too large");
    // distinct sizes, first-occurrence order; a repeated size repeats its row
    std::vector<int> uniq;
    for (int i = 0; i < n_sizes; ++i)
        if (std::find(uniq.begin(), uniq.end(), sizes[i]) == uniq.end()) uniq.push_back(sizes[i]);
    std::vector<std::vector<double>> obs(uniq.size(), std::vector<double>((size_t)t_steps * 7));
    // one batch holds up to 16 distinct sizes; the streams are keyed by (seed,
    // L), so results do not depend on this grouping
    for (size_t g = 0; g < uniq.size(); g += 16) {
        const size_t ge = std::min(uniq.size(), g + 16);
        std::vector<int> grp(uniq.begin() + g, uniq.begin() + ge);
        std::vector<std::vector<double>> part(grp.size());
        for (size_t s = 0; s < grp.size(); ++s) part[s].swap(obs[g + s]);
        const int rc = anneal_group(grp, dim, t_min, t_max, t_steps, J, hfield, warmup, samples,
                                    seed, part);
        for (size_t s = 0; s < grp.size(); ++s) part[s].swap(obs[g + s]);
        if (rc) return rc;
    }
    for (int i = 0; i < n_sizes; ++i) {
        const size_t u = (size_t)(std::find(uniq.begin(), uniq.end(), sizes[i]) - uniq.begin());
        memcpy(out + (size_t)i * t_steps * 7, obs[u].data(), sizeof(double) * t_steps * 7);
    }
    return ISG_OK;
}
