// coarsening — drop-in for the reference's `coarsening --gpu`
// (src/bin/coarsening.rs with src/cuda/coarsening_gpu.rs) on libisinggb.
//
// Same flags and defaults (coarsening.rs:45-123 over CoarseningConfig::default,
// src/coarsening.rs:36-50), the same help/unknown-flag/parse behaviour
// (cli.rs), the same validation messages (coarsening.rs:125-137), the same
// progress lines and the same output <outdir>/coarsening_N<n>_T<t_quench:.2>.csv
// with header "t,rho" and rho with 8 decimals (coarsening.rs:139-160).  The
// protocol itself is isg_coarsening.
//
// Differences by design:
//   * this drop-in provides the GPU path only: without --gpu (the CPU
//     run_coarsening) it exits with an error;
//   * odd sizes are rejected (the reference kernel's thread->site mapping is
//     wrong for odd n, kernels.cu:22-29); --geometry is parsed and validated
//     but, as in the reference GPU path, the lattice is always cubic;
//   * the help text lists the defaults the program actually uses.
#include <string>
#include <vector>

#include "isg.h"
#include "rust_cli.hpp"

namespace {

const char* kUsage =
    "coarsening — domain coarsening after a quench (GB300 GPU path)\n"
    "\n"
    "USAGE:\n"
    "    coarsening --gpu [OPTIONS]\n"
    "\n"
    "OPTIONS:\n"
    "    --n <N>              Lattice size per dimension, even [default: 30]\n"
    "    --geometry <TYPE>    square, triangular or cubic; the GPU lattice is cubic\n"
    "    --j <J>              Coupling constant [default: 1]\n"
    "    --t-high <T>         Equilibration temperature before the quench [default: 10]\n"
    "    --t-quench <T>       Quench temperature [default: 0.5]\n"
    "    --warmup <N>         Sweeps at T_high [default: 200]\n"
    "    --steps <N>          Sweeps after the quench [default: 50000]\n"
    "    --sample-every <N>   Domain-wall density every N sweeps [default: 100]\n"
    "    --seed <N>           Seed of the Philox streams [default: 42]\n"
    "    --gpu                Run on the GPU (required: only the GPU path is provided)\n"
    "    --outdir <DIR>       Output directory [default: analysis/data]\n"
    "    --help, -h           Show this help message";

const std::vector<std::string> kKnownFlags = {
    "--n",    "--geometry",     "--j",    "--t-high", "--t-quench", "--warmup",
    "--steps", "--sample-every", "--seed", "--gpu",    "--outdir",   "--help"};

}  // namespace

int main(int argc, char** argv) {
    using namespace rcli;
    check_help(argc, argv, kUsage);
    warn_unknown_flags(argc, argv, kKnownFlags);

    uint64_t n = 30, warmup = 200, steps = 50000, sample_every = 100, seed = 42;
    double j = 1.0, t_high = 10.0, t_quench = 0.5;
    std::string geometry = "Cubic3D", outdir = "analysis/data";
    bool use_gpu = false;

    int i = 1;
    while (i < argc) {
        const std::string f = argv[i];
        if (f == "--n") n = parse_arg<uint64_t>(argc, argv, i, "--n"), i += 2;
        else if (f == "--geometry") {
            const std::string g = get_arg(argc, argv, i, "--geometry");
            if (g == "cubic") geometry = "Cubic3D";
            else if (g == "triangular") geometry = "Triangular2D";
            else if (g == "square") geometry = "Square2D";
            else die("Error: unknown geometry '" + g + "' (expected: square, triangular, cubic)");
            i += 2;
        } else if (f == "--j") j = parse_arg<double>(argc, argv, i, "--j"), i += 2;
        else if (f == "--t-high") t_high = parse_arg<double>(argc, argv, i, "--t-high"), i += 2;
        else if (f == "--t-quench") t_quench = parse_arg<double>(argc, argv, i, "--t-quench"), i += 2;
        else if (f == "--warmup") warmup = parse_arg<uint64_t>(argc, argv, i, "--warmup"), i += 2;
        else if (f == "--steps") steps = parse_arg<uint64_t>(argc, argv, i, "--steps"), i += 2;
        else if (f == "--sample-every")
            sample_every = parse_arg<uint64_t>(argc, argv, i, "--sample-every"), i += 2;
        else if (f == "--seed") seed = parse_arg<uint64_t>(argc, argv, i, "--seed"), i += 2;
        else if (f == "--outdir") outdir = get_arg(argc, argv, i, "--outdir"), i += 2;
        else if (f == "--gpu") use_gpu = true, i += 1;
        else i += 1;
    }

    // validation, in the reference's order (coarsening.rs:125-137)
    if (n < 2) die("Error: --n must be at least 2 (got " + std::to_string(n) + ")");
    if (t_quench <= 0.0 || t_high <= 0.0) die("Error: temperatures must be positive");
    if (steps == 0) die("Error: --steps must be at least 1");
    if (sample_every == 0) die("Error: --sample-every must be at least 1");
    if (!use_gpu) die("Error: this drop-in provides only the GPU path; pass --gpu");
    if (n > 1024 || (n & 1))
        die("Error: size " + std::to_string(n) +
            " unsupported: the checkerboard update needs an even size in 2..1024");
    if (steps > ((uint64_t)1 << 40) || warmup > ((uint64_t)1 << 40) ||
        sample_every > ((uint64_t)1 << 30))
        die("Error: --steps and --warmup must be at most 2^40, --sample-every at most 2^30");

    std::string err;
    if (!mkdirs(outdir, &err)) panic_expect("src/bin/coarsening.rs", "failed to create outdir", err);
    fprintf(stderr, "Coarsening: N=%llu, geometry=%s, T_quench=%s, steps=%llu [GPU]\n",
            (unsigned long long)n, geometry.c_str(), rust_f64(t_quench).c_str(),
            (unsigned long long)steps);
    fprintf(stderr, "GPU mode: CUDA checkerboard Metropolis\n");
    const int64_t pts = (int64_t)((steps - 1) / sample_every + 1);
    std::vector<int64_t> st((size_t)pts);
    std::vector<double> rho((size_t)pts);
    int64_t got = 0;
    if (isg_coarsening((int)n, j, t_high, t_quench, (int64_t)warmup, (int64_t)steps,
                       (int64_t)sample_every, seed, st.data(), rho.data(), pts, &got) != ISG_OK)
        panic_expect("src/cuda/coarsening_gpu.rs", "GPU step failed", isg_last_error());

    char buf[64];
    snprintf(buf, sizeof buf, "%.2f", t_quench);
    const std::string path =
        join_path(outdir, "coarsening_N" + std::to_string(n) + "_T" + buf + ".csv");
    std::string csv = "t,rho\n";
    for (int64_t k = 0; k < got; ++k) {
        snprintf(buf, sizeof buf, "%lld,%.8f\n", (long long)st[k], rho[k]);
        csv += buf;
    }
    FILE* fp = fopen(path.c_str(), "w");
    if (!fp) panic_expect("src/bin/coarsening.rs", "failed to write CSV", strerror(errno));
    fwrite(csv.data(), 1, csv.size(), fp);
    fclose(fp);
    fprintf(stderr, "Wrote %s\n", path.c_str());
    return 0;
}
