// gpu_fss — drop-in for the reference's src/bin/gpu_fss.rs on libisinggb.
//
// Same flags and defaults (gpu_fss.rs:23-96, unknown flags ignored, malformed
// --sizes entries dropped), the same validation messages and exit codes
// (cli.rs:10-28,86-107; gpu_fss.rs:103-109,158-161), the same CSV files:
//   gpu_fss_{model}_N{n}_timeseries.csv  "temp_idx,E,M" rows, {:.8}
//   gpu_fss_{model}_N{n}_summary.csv     jackknife table, {:.6}
// (gpu_fss.rs:212-320, 476-580).  Differences by design:
//   * all sizes and replicas run together in one batch (one persistent kernel
//     per half-sweep) instead of one size after another;
//   * spins start from the seeded Philox stream (the reference's start is
//     unseeded) and the exchange uses the Philox EXCH stream instead of a host
//     Xoshiro256++ (gpu_fss.rs:197);
//   * continuous models propose inside a cone of half-angle --delta
//     (heisenberg/metropolis.rs:54-69; XY: angle step uniform in [-delta,
//     delta]) and renormalise every --renorm-every sweeps (new flag,
//     default 100);
//   * odd or repeated sizes are rejected/merged (the reference kernel
//     mapping is wrong for odd N, kernels.cu:28).
// Two new flags for the reweighting consumers:
//   --timeseries-format csv|bin|both  (default csv) also or instead writes
//     gpu_fss_{model}_N{n}_timeseries.bin, the exact FP64 records in the
//     binary layout of include/isg.h (isg_ts_*);
//   --histograms (ising) accumulates exact energy histograms on the device
//     and writes gpu_fss_ising_N{n}_hist.bin (isg_ising_hist_*,
//     isg_hist_write).
#include <algorithm>
#include <string>
#include <vector>

#include "isg.h"
#include "rust_cli.hpp"

namespace {

using rcli::die;
using rcli::get_arg;
using rcli::join_path;
using rcli::mkdirs;
using rcli::parse_arg;
using rcli::rust_f64;

[[noreturn]] void panic_expect(const char* what, const std::string& err) {
    rcli::panic_expect("src/bin/gpu_fss.rs", what, err);
}

std::vector<double> linspace(double a, double b, uint64_t n) {
    std::vector<double> t;
    if (n == 1) return {a};
    for (uint64_t i = 0; i < n; ++i) t.push_back(a + (b - a) * (double)i / (double)(n - 1));
    return t;
}

struct Series {
    std::vector<double> e, m;
};

void write_summary(const std::string& path, const std::vector<double>& temps,
                   const std::vector<Series>& ts, double n3) {
    std::string csv = "T,E,E_err,M,M_err,M2,M2_err,M4,M4_err,Cv,Cv_err,chi,chi_err\n";
    char buf[64];
    for (size_t t = 0; t < ts.size(); ++t) {
        if (ts[t].e.empty()) continue;
        const double beta = 1.0 / temps[t];
        const int nb = (int)std::min<size_t>(20, ts[t].e.size());
        double obs[12];
        isg_jackknife(ts[t].e.data(), ts[t].m.data(), (int64_t)ts[t].e.size(), beta, n3, nb, obs);
        snprintf(buf, sizeof buf, "%.6f", temps[t]);
        csv += buf;
        for (int k = 0; k < 12; ++k) {
            snprintf(buf, sizeof buf, ",%.6f", obs[k]);
            csv += buf;
        }
        csv += "\n";
    }
    FILE* f = fopen(path.c_str(), "w");
    if (!f) panic_expect("write summary failed", strerror(errno));
    fwrite(csv.data(), 1, csv.size(), f);
    fclose(f);
    fprintf(stderr, "  Wrote %s\n", path.c_str());
}

struct Run {
    std::string model;
    std::vector<int> sizes;
    double tmin, tmax;
    uint64_t R, warmup, samples, ee, seed, n_or, me, renorm;
    std::string outdir;
    double delta;
    std::string ts_format = "csv";
    bool hist = false;
};

FILE* open_ts(const std::string& path) {
    FILE* f = fopen(path.c_str(), "w");
    if (!f) panic_expect("create timeseries file failed", strerror(errno));
    fprintf(f, "temp_idx,E,M\n");
    return f;
}

// The timeseries of one size in the requested formats.
struct TsOut {
    FILE* csv = nullptr;
    isg_ts* bin = nullptr;
    std::string csv_path, bin_path;
    std::vector<int32_t> bt, br;
    std::vector<double> be, bm;
    char line[128];

    void open(const Run& a, int n, const std::vector<double>& temps) {
        const std::string stem = join_path(a.outdir, "gpu_fss_" + a.model + "_N" + std::to_string(n) +
                                                         "_timeseries");
        if (a.ts_format != "bin") {
            csv_path = stem + ".csv";
            csv = open_ts(csv_path);
        }
        if (a.ts_format != "csv") {
            bin_path = stem + ".bin";
            const int model = a.model == "ising" ? 0 : a.model == "heisenberg" ? 1 : 2;
            if (isg_ts_open(&bin, bin_path.c_str(), model, n, temps.data(), (int)temps.size()) !=
                ISG_OK)
                panic_expect("create timeseries file failed", isg_last_error());
        }
    }
    void add(int t, int r, double e, double m) {
        if (csv) {
            int k = snprintf(line, sizeof line, "%d,%.8f,%.8f\n", t, e, m);
            fwrite(line, 1, (size_t)k, csv);
        }
        if (bin) {
            bt.push_back(t);
            br.push_back(r);
            be.push_back(e);
            bm.push_back(m);
        }
    }
    void flush() {
        if (bin && !bt.empty()) {
            if (isg_ts_append(bin, bt.data(), br.data(), be.data(), bm.data(), (int64_t)bt.size()) !=
                ISG_OK)
                panic_expect("write timeseries row failed", isg_last_error());
            bt.clear();
            br.clear();
            be.clear();
            bm.clear();
        }
    }
    void close() {
        flush();
        if (csv) {
            fclose(csv);
            fprintf(stderr, "  Wrote %s\n", csv_path.c_str());
        }
        if (bin) {
            if (isg_ts_close(bin) != ISG_OK)
                panic_expect("flush timeseries failed", isg_last_error());
            fprintf(stderr, "  Wrote %s\n", bin_path.c_str());
        }
        csv = nullptr;
        bin = nullptr;
    }
};

void empty_outputs(const Run& a, int n) {
    // --replicas 0: header-only files, as the reference loops write them
    std::vector<double> temps;
    TsOut out;
    out.open(a, n, temps);
    out.close();
    std::vector<Series> none;
    write_summary(join_path(a.outdir, "gpu_fss_" + a.model + "_N" + std::to_string(n) +
                                          "_summary.csv"),
                  temps, none, (double)n * n * n);
}

void run_ising(const Run& a) {
    const std::vector<double> temps = linspace(a.tmin, a.tmax, a.R);
    const int R = (int)a.R;
    const int NS = (int)a.sizes.size();
    if (R == 0) {
        for (int n : a.sizes) empty_outputs(a, n);
        return;
    }
    for (int n : a.sizes) fprintf(stderr, "  N=%d: creating %d replicas...\n", n, R);
    isg_ising* h = nullptr;
    if (isg_ising_create(&h, a.sizes.data(), NS, R, 3, a.seed) != ISG_OK)
        panic_expect("failed to create GPU lattice", isg_last_error());
    std::vector<double> all_t;
    for (int s = 0; s < NS; ++s) all_t.insert(all_t.end(), temps.begin(), temps.end());
    if (isg_ising_set_temperatures(h, all_t.data(), 1.0, 0.0) != ISG_OK)
        panic_expect("GPU step failed", isg_last_error());
    fprintf(stderr, "  warming up %llu sweeps...\n", (unsigned long long)a.warmup);
    for (uint64_t w = 0; w < a.warmup;) {
        uint64_t chunk = std::min<uint64_t>(1000 - w % 1000, a.warmup - w);
        if (isg_ising_step(h, (int64_t)chunk) != ISG_OK)
            panic_expect("GPU step failed", isg_last_error());
        w += chunk;
        if (w % 1000 == 0) {
            isg_ising_sync(h);
            fprintf(stderr, "    warmup %llu/%llu\n", (unsigned long long)w,
                    (unsigned long long)a.warmup);
        }
    }
    if (isg_ising_reset_sampling(h) != ISG_OK) panic_expect("GPU step failed", isg_last_error());
    if (a.hist && isg_ising_hist_enable(h, 1) != ISG_OK)
        panic_expect("GPU step failed", isg_last_error());
    std::vector<TsOut> tsf(NS);
    for (int s = 0; s < NS; ++s) tsf[s].open(a, a.sizes[s], temps);
    if (a.ee == 0) {
        fprintf(stderr, "thread 'main' panicked at src/bin/gpu_fss.rs:245:30:\n"
                        "attempt to calculate the remainder with a divisor of zero\n");
        exit(101);
    }
    std::vector<std::vector<Series>> ts(NS, std::vector<Series>(R));
    const int RT = NS * R;
    fprintf(stderr, "  sampling %llu sweeps with PT exchange every %llu...\n",
            (unsigned long long)a.samples, (unsigned long long)a.ee);
    const uint64_t chunk_sweeps = 10000;
    std::vector<int32_t> rt;
    std::vector<int64_t> rb, rm;
    for (uint64_t done = 0; done < a.samples;) {
        uint64_t n = std::min<uint64_t>(chunk_sweeps - done % chunk_sweeps, a.samples - done);
        uint64_t rows = n / a.me + 2;
        rt.assign(rows * RT, 0);
        rb.assign(rows * RT, 0);
        rm.assign(rows * RT, 0);
        int64_t got = 0;
        if (isg_ising_pt_run(h, (int64_t)n, (int)std::min<uint64_t>(a.ee, 1u << 30),
                             (int)std::min<uint64_t>(a.me, 1u << 30), rt.data(), rb.data(),
                             rm.data(), (int64_t)rows, &got) != ISG_OK)
            panic_expect("GPU step failed", isg_last_error());
        for (int s = 0; s < NS; ++s) {
            const double n3 = (double)a.sizes[s] * a.sizes[s] * a.sizes[s];
            for (int64_t row = 0; row < got; ++row)
                for (int r = 0; r < R; ++r) {
                    const size_t o = (size_t)row * RT + (size_t)s * R + r;
                    const int t = rt[o];
                    const double e_per = -(double)rb[o] / n3;
                    const double m_per = fabs((double)rm[o]) / n3;
                    ts[s][t].e.push_back(e_per);
                    ts[s][t].m.push_back(m_per);
                    tsf[s].add(t, r, e_per, m_per);
                }
            tsf[s].flush();
        }
        done += n;
        if (done % 10000 == 0)
            fprintf(stderr, "    sweep %llu/%llu\n", (unsigned long long)done,
                    (unsigned long long)a.samples);
    }
    for (int s = 0; s < NS; ++s) {
        tsf[s].close();
        const double n3 = (double)a.sizes[s] * a.sizes[s] * a.sizes[s];
        write_summary(join_path(a.outdir, "gpu_fss_ising_N" + std::to_string(a.sizes[s]) +
                                              "_summary.csv"),
                      temps, ts[s], n3);
        if (a.hist) {
            std::vector<int64_t> lo(R), nb(R);
            std::vector<uint64_t> cnt;
            for (int t = 0; t < R; ++t) {
                if (isg_ising_hist_range(h, s, t, &lo[t], &nb[t]) != ISG_OK)
                    panic_expect("GPU step failed", isg_last_error());
                const size_t at = cnt.size();
                cnt.resize(at + 4 * (size_t)nb[t]);
                if (nb[t] > 0 && isg_ising_hist_read(h, s, t, lo[t], nb[t], cnt.data() + at) != ISG_OK)
                    panic_expect("GPU step failed", isg_last_error());
            }
            const std::string hp = join_path(a.outdir, "gpu_fss_ising_N" +
                                                           std::to_string(a.sizes[s]) + "_hist.bin");
            if (isg_hist_write(hp.c_str(), 3, a.sizes[s], 1.0, temps.data(), R, lo.data(),
                               nb.data(), cnt.data()) != ISG_OK)
                panic_expect("write histogram file failed", isg_last_error());
            fprintf(stderr, "  Wrote %s\n", hp.c_str());
        }
    }
    isg_ising_destroy(h);
}

void run_continuous(const Run& a, int n_comp) {
    const std::vector<double> temps = linspace(a.tmin, a.tmax, a.R);
    const int R = (int)a.R;
    const int NS = (int)a.sizes.size();
    if (R == 0) {
        for (int n : a.sizes) empty_outputs(a, n);
        return;
    }
    for (int n : a.sizes)
        fprintf(stderr, "  N=%d: creating %d %s replicas...\n", n, R, a.model.c_str());
    isg_cont* h = nullptr;
    if (isg_cont_create(&h, a.sizes.data(), NS, R, n_comp, a.seed) != ISG_OK)
        panic_expect("failed to create continuous GPU lattice", isg_last_error());
    std::vector<double> all_t;
    for (int s = 0; s < NS; ++s) all_t.insert(all_t.end(), temps.begin(), temps.end());
    if (isg_cont_set_temperatures(h, all_t.data(), 1.0) != ISG_OK)
        panic_expect("sweep failed", isg_last_error());
    fprintf(stderr, "  warming up %llu sweeps...\n", (unsigned long long)a.warmup);
    for (uint64_t w = 0; w < a.warmup;) {
        uint64_t chunk = std::min<uint64_t>(1000 - w % 1000, a.warmup - w);
        if (isg_cont_sweep(h, (int64_t)chunk, a.delta, (int)a.n_or) != ISG_OK)
            panic_expect("sweep failed", isg_last_error());
        w += chunk;
        if (w % 1000 == 0) {
            isg_cont_sync(h);
            fprintf(stderr, "    warmup %llu/%llu\n", (unsigned long long)w,
                    (unsigned long long)a.warmup);
        }
    }
    if (isg_cont_reset_sampling(h) != ISG_OK) panic_expect("sweep failed", isg_last_error());
    std::vector<TsOut> tsf(NS);
    for (int s = 0; s < NS; ++s) tsf[s].open(a, a.sizes[s], temps);
    if (a.ee == 0) {
        fprintf(stderr, "thread 'main' panicked at src/bin/gpu_fss.rs:504:30:\n"
                        "attempt to calculate the remainder with a divisor of zero\n");
        exit(101);
    }
    std::vector<std::vector<Series>> ts(NS, std::vector<Series>(R));
    const int RT = NS * R;
    fprintf(stderr, "  sampling %llu sweeps with PT (measure every %llu)...\n",
            (unsigned long long)a.samples, (unsigned long long)a.me);
    std::vector<int32_t> rt;
    std::vector<double> re, rmv, rh;
    for (uint64_t done = 0; done < a.samples;) {
        uint64_t n = std::min<uint64_t>(10000 - done % 10000, a.samples - done);
        uint64_t rows = n / a.me + 2;
        rt.assign(rows * RT, 0);
        re.assign(rows * RT, 0.0);
        rmv.assign(rows * RT * 3, 0.0);
        rh.assign(rows * RT * 6, 0.0);
        int64_t got = 0;
        if (isg_cont_pt_run(h, (int64_t)n, (int)std::min<uint64_t>(a.ee, 1u << 30),
                            (int)std::min<uint64_t>(a.me, 1u << 30), a.delta, (int)a.n_or,
                            (int)std::min<uint64_t>(a.renorm, 1u << 30), rt.data(), re.data(),
                            rmv.data(), rh.data(), (int64_t)rows, &got) != ISG_OK)
            panic_expect("sweep failed", isg_last_error());
        for (int s = 0; s < NS; ++s) {
            const double n3 = (double)a.sizes[s] * a.sizes[s] * a.sizes[s];
            for (int64_t row = 0; row < got; ++row)
                for (int r = 0; r < R; ++r) {
                    const size_t o = (size_t)row * RT + (size_t)s * R + r;
                    const int t = rt[o];
                    const double* m = &rmv[o * 3];
                    const double e_per = re[o] / n3;
                    const double m_abs = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) / n3;
                    ts[s][t].e.push_back(e_per);
                    ts[s][t].m.push_back(m_abs);
                    tsf[s].add(t, r, e_per, m_abs);
                }
            tsf[s].flush();
        }
        done += n;
        if (done % 10000 == 0)
            fprintf(stderr, "    sweep %llu/%llu\n", (unsigned long long)done,
                    (unsigned long long)a.samples);
    }
    for (int s = 0; s < NS; ++s) {
        tsf[s].close();
        const double n3 = (double)a.sizes[s] * a.sizes[s] * a.sizes[s];
        write_summary(join_path(a.outdir, "gpu_fss_" + a.model + "_N" +
                                              std::to_string(a.sizes[s]) + "_summary.csv"),
                      temps, ts[s], n3);
    }
    isg_cont_destroy(h);
}

}  // namespace

int main(int argc, char** argv) {
    Run a;
    a.model = "ising";
    std::string sizes_str = "8,16,32,64";
    a.tmin = 4.4;
    a.tmax = 4.6;
    a.R = 20;
    a.warmup = 5000;
    a.samples = 100000;
    a.ee = 10;
    a.seed = 42;
    a.outdir = "analysis/data";
    a.delta = 0.5;
    a.n_or = 5;
    a.me = 1;
    a.renorm = 100;
    int i = 1;
    while (i < argc) {
        std::string f = argv[i];
        if (f == "--model") a.model = get_arg(argc, argv, i, "--model"), i += 2;
        else if (f == "--sizes") sizes_str = get_arg(argc, argv, i, "--sizes"), i += 2;
        else if (f == "--tmin") a.tmin = parse_arg<double>(argc, argv, i, "--tmin"), i += 2;
        else if (f == "--tmax") a.tmax = parse_arg<double>(argc, argv, i, "--tmax"), i += 2;
        else if (f == "--replicas") a.R = parse_arg<uint64_t>(argc, argv, i, "--replicas"), i += 2;
        else if (f == "--warmup") a.warmup = parse_arg<uint64_t>(argc, argv, i, "--warmup"), i += 2;
        else if (f == "--samples") a.samples = parse_arg<uint64_t>(argc, argv, i, "--samples"), i += 2;
        else if (f == "--exchange-every")
            a.ee = parse_arg<uint64_t>(argc, argv, i, "--exchange-every"), i += 2;
        else if (f == "--seed") a.seed = parse_arg<uint64_t>(argc, argv, i, "--seed"), i += 2;
        else if (f == "--outdir") a.outdir = get_arg(argc, argv, i, "--outdir"), i += 2;
        else if (f == "--delta") a.delta = parse_arg<double>(argc, argv, i, "--delta"), i += 2;
        else if (f == "--overrelax") a.n_or = parse_arg<uint64_t>(argc, argv, i, "--overrelax"), i += 2;
        else if (f == "--measure-every")
            a.me = parse_arg<uint64_t>(argc, argv, i, "--measure-every"), i += 2;
        else if (f == "--renorm-every")
            a.renorm = parse_arg<uint64_t>(argc, argv, i, "--renorm-every"), i += 2;
        else if (f == "--timeseries-format")
            a.ts_format = get_arg(argc, argv, i, "--timeseries-format"), i += 2;
        else if (f == "--histograms") a.hist = true, i += 1;
        else i += 1;
    }
    // sizes: comma-separated, trimmed, malformed entries dropped (gpu_fss.rs:98-101)
    std::vector<int> sizes_all = rcli::parse_sizes(sizes_str, true);
    // validate_temp_range / validate_samples (cli.rs:86-107), gpu_fss.rs:103-109
    if (a.tmin <= 0.0) die("Error: --tmin must be positive (got " + rust_f64(a.tmin) + ")");
    if (a.tmax <= 0.0) die("Error: --tmax must be positive (got " + rust_f64(a.tmax) + ")");
    if (a.tmin >= a.tmax)
        die("Error: --tmin (" + rust_f64(a.tmin) + ") must be less than --tmax (" +
            rust_f64(a.tmax) + ")");
    if (a.samples == 0) die("Error: --samples must be at least 1");
    if (a.warmup == 0) die("Error: --warmup must be at least 1");
    if (a.me == 0) die("Error: --measure-every must be at least 1");
    if (a.ts_format != "csv" && a.ts_format != "bin" && a.ts_format != "both")
        die("Error: --timeseries-format must be csv, bin or both");
    if (a.hist && a.model != "ising")
        die("Error: --histograms needs --model ising (exact energy bins)");
    std::string err;
    if (!mkdirs(a.outdir, &err)) panic_expect("failed to create outdir", err);
    std::string sz = "[";
    for (size_t k = 0; k < sizes_all.size(); ++k)
        sz += (k ? ", " : "") + std::to_string(sizes_all[k]);
    sz += "]";
    fprintf(stderr, "GPU FSS: model=%s, sizes=%s, T=%s..%s, replicas=%llu\n", a.model.c_str(),
            sz.c_str(), rust_f64(a.tmin).c_str(), rust_f64(a.tmax).c_str(),
            (unsigned long long)a.R);
    if (a.model != "ising" && a.model != "xy" && a.model != "heisenberg")
        die("Error: --model must be ising, xy, or heisenberg");
    for (int n : sizes_all) {
        if (n < 2 || n > 1024 || (n & 1))
            die("Error: size " + std::to_string(n) +
                " unsupported: the checkerboard update needs an even size in 2..1024");
        if (std::find(a.sizes.begin(), a.sizes.end(), n) == a.sizes.end()) a.sizes.push_back(n);
    }
    if (a.R > 1024) die("Error: --replicas must be at most 1024");
    if (a.sizes.size() > 16) die("Error: at most 16 distinct sizes per run");
    if (a.sizes.empty()) return 0;
    if (a.model == "ising") run_ising(a);
    else run_continuous(a, a.model == "xy" ? 2 : 3);
    return 0;
}
