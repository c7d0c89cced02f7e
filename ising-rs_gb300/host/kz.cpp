// kz — drop-in for the reference's `kz --gpu` (src/bin/kz.rs with
// src/cuda/kz_gpu.rs) on libisinggb.
//
// Same flags and defaults (kz.rs:59-146), the same help/unknown-flag/parse
// behaviour (cli.rs), the same validation messages in the same order
// (kz.rs:148-171), the same log-spaced tau_q values (kz.rs:173-185: rounded
// exp of a linear grid in ln tau), the same progress lines and the same output
// <outdir>/kz_N<n>.csv with header "tau_q,rho,rho_err,n_trials" and rho,
// rho_err with 8 decimals (kz.rs:240-249).  The protocol itself is
// isg_kz_sweep.
//
// Differences by design:
//   * this drop-in provides the GPU path only: without --gpu (the CPU run_kz_sweep)
//     it exits with an error;
//   * every tau_q's trials run as one batch and all tau_q values run at the
//     same time, so the per-tau_q progress lines come out together; trial t
//     of tau_q uses replica t of the stream keyed by seed + tau_q (the
//     reference seeds it with seed + tau_q + t);
//   * the help text lists the defaults the program actually uses.
#include <math.h>

#include <string>
#include <vector>

#include "isg.h"
#include "rust_cli.hpp"

namespace {

const char* kUsage =
    "kz — Kibble-Zurek quench sweeps (GB300 GPU path)\n"
    "\n"
    "USAGE:\n"
    "    kz --gpu [OPTIONS]\n"
    "\n"
    "OPTIONS:\n"
    "    --n <N>                   Lattice size per dimension [default: 20]\n"
    "    --geometry <TYPE>         square, triangular or cubic; --gpu needs cubic [default: cubic]\n"
    "    --j <J>                   Coupling constant [default: 1]\n"
    "    --t-start <T>             Ramp start temperature [default: 6]\n"
    "    --t-end <T>               Ramp end temperature [default: 1]\n"
    "    --tau-min <N>             Shortest quench time in sweeps [default: 100]\n"
    "    --tau-max <N>             Longest quench time in sweeps [default: 100000]\n"
    "    --tau-steps <N>           Number of log-spaced quench times [default: 20]\n"
    "    --trials <N>              Independent trials per quench time [default: 5]\n"
    "    --warmup-sweeps <N>       Sweeps at the start temperature [default: 200]\n"
    "    --freeze-sweeps <N>       Sweeps at the freeze temperature after the ramp [default: 0]\n"
    "    --freeze-temperature <T>  Freeze temperature [default: 0.01]\n"
    "    --seed <N>                Seed of the Philox streams [default: 42]\n"
    "    --gpu                     Run on the GPU (required: only the GPU path is provided)\n"
    "    --outdir <DIR>            Output directory [default: analysis/data]\n"
    "    --help, -h                Show this help message";

const std::vector<std::string> kKnownFlags = {
    "--n",        "--geometry", "--j",         "--t-start",       "--t-end",
    "--tau-min",  "--tau-max",  "--tau-steps", "--trials",        "--warmup-sweeps",
    "--freeze-sweeps", "--freeze-temperature", "--seed", "--gpu", "--outdir", "--help"};

// Rust {:.4} of a positive-or-negative f64
std::string fixed(double x, int prec) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.*f", prec, x);
    return buf;
}

}  // namespace

int main(int argc, char** argv) {
    using namespace rcli;
    check_help(argc, argv, kUsage);
    warn_unknown_flags(argc, argv, kKnownFlags);

    uint64_t n = 20, tau_min = 100, tau_max = 100000, tau_steps = 20, n_trials = 5;
    uint64_t warmup = 200, freeze = 0, seed = 42;
    double j = 1.0, t_start = 6.0, t_end = 1.0, freeze_t = 0.01;
    std::string geometry = "cubic", outdir = "analysis/data";
    bool use_gpu = false;

    int i = 1;
    while (i < argc) {
        const std::string f = argv[i];
        if (f == "--n") n = parse_arg<uint64_t>(argc, argv, i, "--n"), i += 2;
        else if (f == "--geometry") {
            geometry = get_arg(argc, argv, i, "--geometry");
            if (geometry != "cubic" && geometry != "triangular" && geometry != "square")
                die("Error: unknown geometry '" + geometry +
                    "' (expected: square, triangular, cubic)");
            i += 2;
        } else if (f == "--j") j = parse_arg<double>(argc, argv, i, "--j"), i += 2;
        else if (f == "--t-start") t_start = parse_arg<double>(argc, argv, i, "--t-start"), i += 2;
        else if (f == "--t-end") t_end = parse_arg<double>(argc, argv, i, "--t-end"), i += 2;
        else if (f == "--tau-min") tau_min = parse_arg<uint64_t>(argc, argv, i, "--tau-min"), i += 2;
        else if (f == "--tau-max") tau_max = parse_arg<uint64_t>(argc, argv, i, "--tau-max"), i += 2;
        else if (f == "--tau-steps")
            tau_steps = parse_arg<uint64_t>(argc, argv, i, "--tau-steps"), i += 2;
        else if (f == "--trials") n_trials = parse_arg<uint64_t>(argc, argv, i, "--trials"), i += 2;
        else if (f == "--warmup-sweeps")
            warmup = parse_arg<uint64_t>(argc, argv, i, "--warmup-sweeps"), i += 2;
        else if (f == "--freeze-sweeps")
            freeze = parse_arg<uint64_t>(argc, argv, i, "--freeze-sweeps"), i += 2;
        else if (f == "--freeze-temperature")
            freeze_t = parse_arg<double>(argc, argv, i, "--freeze-temperature"), i += 2;
        else if (f == "--seed") seed = parse_arg<uint64_t>(argc, argv, i, "--seed"), i += 2;
        else if (f == "--outdir") outdir = get_arg(argc, argv, i, "--outdir"), i += 2;
        else if (f == "--gpu") use_gpu = true, i += 1;
        else i += 1;
    }

    // validation, in the reference's order (kz.rs:148-171)
    if (n < 2) die("Error: --n must be at least 2 (got " + std::to_string(n) + ")");
    if (tau_steps == 0) die("Error: --tau-steps must be at least 1");
    if (n_trials == 0) die("Error: --trials must be at least 1");
    if (t_start <= 0.0 || t_end <= 0.0 || freeze_t <= 0.0)
        die("Error: temperatures must be positive");
    if (tau_min == 0 || tau_max == 0 || tau_min > tau_max)
        die("Error: --tau-min must be >= 1 and <= --tau-max");
    if (use_gpu && geometry != "cubic")
        die("Error: --gpu KZ currently supports only --geometry cubic");
    if (!use_gpu) die("Error: this drop-in provides only the GPU path; pass --gpu");
    if (n > 1024 || (n & 1))
        die("Error: size " + std::to_string(n) +
            " unsupported: the checkerboard update needs an even size in 2..1024");
    if (n_trials > 1024) die("Error: --trials must be at most 1024");
    if (tau_steps > 100000) die("Error: --tau-steps must be at most 100000");
    if (tau_max > ((uint64_t)1 << 32) || warmup > ((uint64_t)1 << 32) ||
        freeze > ((uint64_t)1 << 32))
        die("Error: sweep counts must be at most 2^32");

    std::vector<int64_t> taus;
    if (tau_steps == 1) {
        taus.push_back((int64_t)tau_min);
    } else {
        const double lmin = log((double)tau_min), lmax = log((double)tau_max);
        for (uint64_t k = 0; k < tau_steps; ++k) {
            const double lt = lmin + (lmax - lmin) * (double)k / (double)(tau_steps - 1);
            taus.push_back((int64_t)round(exp(lt)));
        }
    }
    const std::string describe = "warmup=" + std::to_string(warmup) +
                                 " sweeps, ramp endpoint measurement, freeze=" +
                                 std::to_string(freeze) + " sweeps at T=" + fixed(freeze_t, 4);
    fprintf(stderr,
            "KZ sweep [GPU]: N=%llu, tau_q=%llu..%llu (%llu steps, log-spaced), %llu trials each\n",
            (unsigned long long)n, (unsigned long long)tau_min, (unsigned long long)tau_max,
            (unsigned long long)tau_steps, (unsigned long long)n_trials);
    fprintf(stderr, "  Ramp: T_start=%s -> T_end=%s; %s\n", rust_f64(t_start).c_str(),
            rust_f64(t_end).c_str(), describe.c_str());
    fprintf(stderr, "  Protocol: ramp T=%s -> T=%s, %s\n", rust_f64(t_start).c_str(),
            rust_f64(t_end).c_str(), describe.c_str());
    for (int64_t t : taus) fprintf(stderr, "  tau_q = %lld ...\n", (long long)t);
    std::vector<double> out(2 * taus.size());
    if (isg_kz_sweep((int)n, j, t_start, t_end, taus.data(), (int)taus.size(), (int)n_trials,
                     (int64_t)warmup, (int64_t)freeze, freeze_t, seed, out.data()) != ISG_OK) {
        fprintf(stderr, "Error: %s\n", isg_last_error());
        return 1;
    }
    for (size_t k = 0; k < taus.size(); ++k)
        fprintf(stderr, "  tau_q = %lld: rho = %.6f +/- %.6f\n", (long long)taus[k], out[2 * k],
                out[2 * k + 1]);

    std::string err;
    if (!mkdirs(outdir, &err)) panic_expect("src/bin/kz.rs", "failed to create outdir", err);
    const std::string path = join_path(outdir, "kz_N" + std::to_string(n) + ".csv");
    std::string csv = "tau_q,rho,rho_err,n_trials\n";
    char buf[128];
    for (size_t k = 0; k < taus.size(); ++k) {
        snprintf(buf, sizeof buf, "%lld,%.8f,%.8f,%llu\n", (long long)taus[k], out[2 * k],
                 out[2 * k + 1], (unsigned long long)n_trials);
        csv += buf;
    }
    FILE* fp = fopen(path.c_str(), "w");
    if (!fp) panic_expect("src/bin/kz.rs", "failed to write CSV", strerror(errno));
    fwrite(csv.data(), 1, csv.size(), fp);
    fclose(fp);
    fprintf(stderr, "Wrote %s\n", path.c_str());
    return 0;
}
