// fss — drop-in for the reference's `fss --gpu` (src/bin/fss.rs with
// src/cuda/fss_gpu.rs) on libisinggb.
//
// Same flags and defaults (fss.rs:59-135 over FssConfig::default,
// src/fss.rs:20-36), the same help/unknown-flag/parse/validation behaviour
// (cli.rs:10-107: messages, exit codes 0/1, `.expect()` panics with 101), the
// same output: one <outdir>/fss_N<n>.csv per size, header "T,E,M,M2,M4,Cv,chi",
// T with 4 decimals and the rest with 6 (fss.rs:190-207), temperatures
// ascending.  The annealing schedule itself is isg_fss_anneal.
//
// Differences by design:
//   * this drop-in provides the GPU path only: without --gpu (the CPU
//     Metropolis/Wolff run_fss), or with --raw (CPU Wolff time series), it
//     exits with an error instead of running on the host;
//   * all sizes anneal together in one batch; size L uses the Philox stream
//     keyed by (seed, L) where the reference seeds size n with seed + n;
//   * odd sizes are rejected (the reference kernel's thread->site mapping is
//     wrong for odd n, kernels.cu:22-29); --geometry is parsed and validated
//     but, as in the reference GPU path, the lattice is always cubic;
//   * the help text lists the defaults the program actually uses.
#include <algorithm>
#include <string>
#include <vector>

#include "isg.h"
#include "rust_cli.hpp"

namespace {

const char* kUsage =
    "fss — finite-size scaling temperature sweeps (GB300 GPU path)\n"
    "\n"
    "USAGE:\n"
    "    fss --gpu [OPTIONS]\n"
    "\n"
    "OPTIONS:\n"
    "    --sizes <N,N,...>    Lattice sizes, even [default: 8,12,16,20,24,28]\n"
    "    --geometry <TYPE>    square, triangular or cubic; the GPU lattice is cubic\n"
    "    --j <J>              Coupling constant [default: 1]\n"
    "    --tmin <T>           Lowest temperature [default: 3.5]\n"
    "    --tmax <T>           Highest temperature [default: 5.5]\n"
    "    --steps <N>          Temperature points, at least 2 [default: 41]\n"
    "    --warmup <N>         Sweeps before measuring, per temperature [default: 500]\n"
    "    --samples <N>        Measured sweeps per temperature [default: 200]\n"
    "    --seed <N>           Seed of the Philox streams [default: 42]\n"
    "    --wolff              Accepted for compatibility (CPU algorithm choice)\n"
    "    --raw                CPU Wolff time series: not provided by this drop-in\n"
    "    --gpu                Run on the GPU (required: only the GPU path is provided)\n"
    "    --outdir <DIR>       Output directory [default: analysis/data]\n"
    "    --help, -h           Show this help message";

const std::vector<std::string> kKnownFlags = {
    "--sizes", "--geometry", "--j",    "--tmin", "--tmax",   "--steps", "--warmup",
    "--samples", "--seed",   "--wolff", "--raw", "--gpu",    "--outdir", "--help"};

}  // namespace

int main(int argc, char** argv) {
    using namespace rcli;
    check_help(argc, argv, kUsage);
    warn_unknown_flags(argc, argv, kKnownFlags);

    std::vector<int> sizes = {8, 12, 16, 20, 24, 28};
    double j = 1.0, t_min = 3.5, t_max = 5.5;
    uint64_t t_steps = 41, warmup = 500, samples = 200, seed = 42;
    std::string outdir = "analysis/data";
    bool use_gpu = false, raw = false;

    int i = 1;
    while (i < argc) {
        const std::string f = argv[i];
        if (f == "--sizes") {
            sizes = parse_sizes(get_arg(argc, argv, i, "--sizes"), false);
            i += 2;
        } else if (f == "--geometry") {
            const std::string g = get_arg(argc, argv, i, "--geometry");
            if (g != "cubic" && g != "triangular" && g != "square")
                die("Error: unknown geometry '" + g + "' (expected: square, triangular, cubic)");
            i += 2;
        } else if (f == "--j") {
            j = parse_arg<double>(argc, argv, i, "--j");
            i += 2;
        } else if (f == "--warmup") {
            warmup = parse_arg<uint64_t>(argc, argv, i, "--warmup");
            i += 2;
        } else if (f == "--samples") {
            samples = parse_arg<uint64_t>(argc, argv, i, "--samples");
            i += 2;
        } else if (f == "--tmin") {
            t_min = parse_arg<double>(argc, argv, i, "--tmin");
            i += 2;
        } else if (f == "--tmax") {
            t_max = parse_arg<double>(argc, argv, i, "--tmax");
            i += 2;
        } else if (f == "--steps") {
            t_steps = parse_arg<uint64_t>(argc, argv, i, "--steps");
            i += 2;
        } else if (f == "--seed") {
            seed = parse_arg<uint64_t>(argc, argv, i, "--seed");
            i += 2;
        } else if (f == "--outdir") {
            outdir = get_arg(argc, argv, i, "--outdir");
            i += 2;
        } else if (f == "--gpu") {
            use_gpu = true;
            i += 1;
        } else if (f == "--raw") {
            raw = true;
            i += 1;
        } else {
            i += 1;  // --wolff and anything else
        }
    }

    // validation, in the reference's order (fss.rs:133-141; cli.rs:70-107)
    if (t_steps < 2) die("Error: --steps must be at least 2 (got " + std::to_string(t_steps) + ")");
    if (t_min <= 0.0) die("Error: --tmin must be positive (got " + rust_f64(t_min) + ")");
    if (t_max <= 0.0) die("Error: --tmax must be positive (got " + rust_f64(t_max) + ")");
    if (t_min >= t_max)
        die("Error: --tmin (" + rust_f64(t_min) + ") must be less than --tmax (" + rust_f64(t_max) +
            ")");
    if (samples == 0) die("Error: --samples must be at least 1");
    if (warmup == 0) die("Error: --warmup must be at least 1");
    for (int n : sizes)
        if (n < 2) die("Error: --n must be at least 2 (got " + std::to_string(n) + ")");
    if (raw && use_gpu) fprintf(stderr, "Warning: --raw mode does not support --gpu; ignoring --gpu\n");
    if (raw) die("Error: --raw (CPU Wolff time series) is not provided by this GPU build");
    if (!use_gpu) die("Error: this drop-in provides only the GPU path; pass --gpu");
    for (int n : sizes)
        if (n > 1024 || (n & 1))
            die("Error: size " + std::to_string(n) +
                " unsupported: the checkerboard update needs an even size in 2..1024");
    if (t_steps > 1000000) die("Error: --steps must be at most 1000000");
    if (warmup > ((uint64_t)1 << 40) || samples > ((uint64_t)1 << 40))
        die("Error: --warmup and --samples must be at most 2^40");

    std::string err;
    if (!mkdirs(outdir, &err)) panic_expect("src/bin/fss.rs", "failed to create outdir", err);

    fprintf(stderr, "GPU mode: CUDA checkerboard Metropolis\n");
    for (int n : sizes) fprintf(stderr, "FSS GPU: N=%d\n", n);
    std::vector<double> obs(sizes.size() * (size_t)t_steps * 7);
    if (!sizes.empty() &&
        isg_fss_anneal(sizes.data(), (int)sizes.size(), 3, t_min, t_max, (int)t_steps, j, 0.0,
                       (int64_t)warmup, (int64_t)samples, seed, obs.data()) != ISG_OK) {
        const std::string e = isg_last_error();
        panic_expect("src/cuda/fss_gpu.rs",
                     e.rfind("isg_ising_create", 0) == 0 ? "failed to create GPU lattice"
                                                         : "GPU measure failed",
                     e);
    }
    char buf[64];
    for (size_t s = 0; s < sizes.size(); ++s) {
        const std::string path = join_path(outdir, "fss_N" + std::to_string(sizes[s]) + ".csv");
        std::string csv = "T,E,M,M2,M4,Cv,chi\n";
        for (uint64_t k = 0; k < t_steps; ++k) {
            const double* o = &obs[(s * t_steps + k) * 7];
            snprintf(buf, sizeof buf, "%.4f", o[0]);
            csv += buf;
            for (int c = 1; c < 7; ++c) {
                snprintf(buf, sizeof buf, ",%.6f", o[c]);
                csv += buf;
            }
            csv += "\n";
        }
        FILE* fp = fopen(path.c_str(), "w");
        if (!fp) panic_expect("src/bin/fss.rs", "failed to write CSV", strerror(errno));
        fwrite(csv.data(), 1, csv.size(), fp);
        fclose(fp);
        fprintf(stderr, "Wrote %s\n", path.c_str());
    }
    return 0;
}
