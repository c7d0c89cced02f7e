// isg_quench.cpp — the quench protocols on the batched Ising engine:
// Kibble-Zurek linear ramps (`kz --gpu`) and coarsening after a sudden quench
// (`coarsening --gpu`).
//
// Reference paths being replaced (faulknco/ising-rs):
//   src/cuda/kz_gpu.rs:9-95          run_kz_gpu / run_kz_sweep_gpu: one
//                                    LatticeGpu per (tau_q, trial), one sweep
//                                    (two launches) per ramp temperature, the
//                                    domain walls counted on the host
//   src/cuda/coarsening_gpu.rs:6-31  run_coarsening_gpu: a full spin copy and
//                                    a host wall count every sample_every sweeps
//   src/kibble_zurek.rs:78-106       linear_ramp_temperature, mean_and_std_err,
//                                    trial_seed
//   src/cuda/lattice_gpu.rs:253-281  domain_wall_density (forward bonds)
//
// Here all trials of one tau_q are the replicas of one batch, every tau_q's
// batch runs its whole schedule (warm-up, ramp, freeze) as one
// isg_ising_run_schedule on its own stream, all of them concurrently, and the
// domain-wall density comes from the exact bond sum B of the forward bonds:
// walls = (3 N^3 - B) / 2, rho = walls / (3 N^3).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "isg.h"

namespace isg {
int fail(int code, const std::string& msg);
}

namespace {

constexpr double kMinTemperature = 0.01;  // kibble_zurek.rs:8

double rho_of_bond(int64_t bond, double bonds) {
    const int64_t nb = (int64_t)bonds;
    const int64_t walls = (nb - bond) / 2;
    return (double)walls / bonds;
}

}  // namespace

extern "C" int isg_kz_sweep(int n, double J, double t_start, double t_end, const int64_t* tau_q,
                            int n_tau, int n_trials, int64_t warmup_sweeps, int64_t freeze_sweeps,
                            double freeze_temperature, uint64_t base_seed, double* out) {
    using isg::fail;
    if (!tau_q || !out || n_tau < 1) return fail(ISG_ERR_ARG, "isg_kz_sweep: no tau_q values");
    if (n_trials < 1 || n_trials > 1024)
        return fail(ISG_ERR_ARG, "isg_kz_sweep: n_trials must be 1..1024");
    if (!(t_start > 0.0) || !(t_end > 0.0) || !(freeze_temperature > 0.0))
        return fail(ISG_ERR_ARG, "isg_kz_sweep: temperatures must be positive");
    if (warmup_sweeps < 0 || freeze_sweeps < 0)
        return fail(ISG_ERR_ARG, "isg_kz_sweep: negative sweep count");
    for (int i = 0; i < n_tau; ++i)
        if (tau_q[i] < 0 || tau_q[i] > ((int64_t)1 << 32))
            return fail(ISG_ERR_ARG, "isg_kz_sweep: tau_q out of range");
    std::vector<isg_ising*> hs(n_tau, nullptr);
    int rc = ISG_OK;
    const double bonds = 3.0 * (double)n * n * n;
    // one batch per tau_q, all running concurrently on their own streams
    for (int i = 0; i < n_tau && rc == 0; ++i) {
        const int64_t tau = tau_q[i];
        // trial t of tau_q uses replica t of the batch keyed by base + tau_q
        // (the reference seeds trial t with base + tau_q + t, kibble_zurek.rs:102-106)
        rc = isg_ising_create(&hs[i], &n, 1, n_trials, 3, base_seed + (uint64_t)tau);
        if (rc) break;
        std::vector<double> temps;
        temps.reserve((size_t)(warmup_sweeps + tau + freeze_sweeps));
        temps.insert(temps.end(), (size_t)warmup_sweeps, t_start);
        for (int64_t step = 0; step < tau; ++step) {
            // linear_ramp_temperature: t_start + (t_end - t_start) * (step + 1) / tau_q
            const double frac = (double)(step + 1) / (double)tau;
            const double t = t_start + (t_end - t_start) * frac;
            temps.push_back(std::max(t, kMinTemperature));
        }
        temps.insert(temps.end(), (size_t)freeze_sweeps,
                     std::max(freeze_temperature, kMinTemperature));
        std::vector<double> t0((size_t)n_trials, t_start);
        rc = isg_ising_set_temperatures(hs[i], t0.data(), J, 0.0);
        if (rc) break;
        if (!temps.empty())
            rc = isg_ising_run_schedule(hs[i], temps.data(), (int64_t)temps.size(), 0, 0, nullptr,
                                        nullptr, 0, nullptr);
    }
    for (int i = 0; i < n_tau && rc == 0; ++i) {
        std::vector<int64_t> b((size_t)n_trials), m((size_t)n_trials);
        rc = isg_ising_measure(hs[i], b.data(), m.data());
        if (rc) break;
        // mean_and_std_err (kibble_zurek.rs:86-100)
        std::vector<double> rho((size_t)n_trials);
        for (int t = 0; t < n_trials; ++t) rho[t] = rho_of_bond(b[t], bonds);
        const double nn = (double)n_trials;
        double sum = 0.0;
        for (double x : rho) sum += x;
        const double mean = sum / nn;
        double err = 0.0;
        if (n_trials > 1) {
            double ss = 0.0;
            for (double x : rho) ss += (x - mean) * (x - mean);
            const double var = ss / (nn - 1.0);
            err = std::sqrt(var) / std::sqrt(nn);
        }
        out[2 * i] = mean;
        out[2 * i + 1] = err;
    }
    for (isg_ising* h : hs)
        if (h) isg_ising_destroy(h);
    return rc;
}

extern "C" int isg_coarsening(int n, double J, double t_high, double t_quench,
                              int64_t warmup_sweeps, int64_t total_steps, int64_t sample_every,
                              uint64_t seed, int64_t* steps_out, double* rho_out,
                              int64_t max_points, int64_t* n_points) {
    using isg::fail;
    if (!(t_high > 0.0) || !(t_quench > 0.0))
        return fail(ISG_ERR_ARG, "isg_coarsening: temperatures must be positive");
    if (warmup_sweeps < 0 || total_steps < 1 || sample_every < 1 || sample_every > (1 << 30))
        return fail(ISG_ERR_ARG, "isg_coarsening: need warmup >= 0, total_steps >= 1 and "
                                 "1 <= sample_every <= 2^30");
    const int64_t pts = (total_steps - 1) / sample_every + 1;
    if (!steps_out || !rho_out || max_points < pts)
        return fail(ISG_ERR_ARG, "isg_coarsening: output arrays hold " +
                                     std::to_string(max_points) + " points, " +
                                     std::to_string(pts) + " needed");
    isg_ising* h = nullptr;
    int rc = isg_ising_create(&h, &n, 1, 1, 3, seed);
    if (rc) return rc;
    std::vector<int64_t> b((size_t)pts), m((size_t)pts);
    int64_t got = 0;
    rc = isg_ising_set_temperatures(h, &t_high, J, 0.0);
    if (!rc && warmup_sweeps > 0)
        rc = isg_ising_run_schedule(h, nullptr, warmup_sweeps, 0, 0, nullptr, nullptr, 0, nullptr);
    const double tq = std::max(t_quench, kMinTemperature);
    if (!rc) rc = isg_ising_set_temperatures(h, &tq, J, 0.0);
    // sample after step `step` when step % sample_every == 0 (coarsening_gpu.rs:21-27)
    if (!rc)
        rc = isg_ising_run_schedule(h, nullptr, total_steps, (int)sample_every, 0, b.data(),
                                    m.data(), pts, &got);
    if (!rc) {
        const double bonds = 3.0 * (double)n * n * n;
        for (int64_t k = 0; k < got; ++k) {
            steps_out[k] = k * sample_every;
            rho_out[k] = rho_of_bond(b[(size_t)k], bonds);
        }
        if (n_points) *n_points = got;
    }
    isg_ising_destroy(h);
    return rc;
}
