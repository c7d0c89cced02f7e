// gpu_jfit — drop-in for the reference's `gpu_jfit` (src/bin/gpu_jfit.rs) on
// libisinggb: parallel tempering of Ising (--model ising), XY (--model xy) or
// Heisenberg (--model heisenberg) spins on a graph read from
// {"n_nodes": N, "edges": [[a, b], ...]} (GraphDef::from_json,
// src/graph.rs:44-79).
//
// Same flags and defaults (gpu_jfit.rs:22-90, unknown flags skipped), the same
// validation messages (gpu_jfit.rs:92-110; cli.rs), the same progress lines and
// the same output <outdir>/gpu_jfit_<model>_<graph>.csv with the reference's
// columns, T with 4 decimals, the rest with 6 and the error columns written as
// 0.0 (gpu_jfit.rs:269-297, 385-411, 498-524): per temperature index the
// running means of e, |m|, m^2, m^4 over every sampling sweep,
// Cv = beta^2 (<e^2> - <e>^2) N and chi = beta (<m^2> - <|m|>^2) N.
//
// Differences by design: the replicas run on the GPU (isg_graph_*,
// isg_cgraph_*) with Philox streams instead of one shared Xoshiro256++:
//   * ising: sites updated colour class by colour class of a greedy proper
//     colouring instead of random-site sweeps;
//   * heisenberg: the same cone Metropolis (half-angle 0.5) by colour class;
//   * xy: one single-cluster Wolff flip per sample, as the reference, grown
//     breadth-first on the device;
// the exchange rule and cadence are the reference's.  Graphs are limited to
// 65536 nodes of degree <= 12 (ising) or 16384 nodes of degree <= 64 (xy,
// heisenberg), and to 1024 replicas; self-loops are rejected.
#include <algorithm>
#include <cctype>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "isg.h"
#include "rust_cli.hpp"

namespace {

[[noreturn]] void panic_expect(const char* what, const std::string& err) {
    rcli::panic_expect("src/bin/gpu_jfit.rs", what, err);
}

// Minimal reader of {"n_nodes": N, "edges": [[a, b], ...]}.
bool parse_graph(const std::string& s, int* n_nodes, std::vector<int32_t>* edges, std::string* err) {
    auto skip = [&](size_t& i) {
        while (i < s.size() && isspace((unsigned char)s[i])) ++i;
    };
    auto read_uint = [&](size_t& i, long long* v) -> bool {
        skip(i);
        if (i >= s.size() || !isdigit((unsigned char)s[i])) return false;
        long long x = 0;
        while (i < s.size() && isdigit((unsigned char)s[i])) {
            x = x * 10 + (s[i] - '0');
            if (x > (1ll << 31)) return false;
            ++i;
        }
        *v = x;
        return true;
    };
    const size_t kn = s.find("\"n_nodes\"");
    if (kn == std::string::npos) {
        *err = "missing n_nodes";
        return false;
    }
    size_t i = s.find(':', kn);
    long long n = 0;
    if (i == std::string::npos || !read_uint(++i, &n)) {
        *err = "n_nodes is not an integer";
        return false;
    }
    *n_nodes = (int)n;
    const size_t ke = s.find("\"edges\"");
    if (ke == std::string::npos) {
        *err = "missing edges";
        return false;
    }
    i = s.find('[', ke);
    if (i == std::string::npos) {
        *err = "edges is not an array";
        return false;
    }
    ++i;
    for (;;) {
        skip(i);
        if (i < s.size() && s[i] == ']') break;
        if (i >= s.size() || s[i] != '[') {
            *err = "edge entry is not a 2-element array";
            return false;
        }
        ++i;
        long long a = 0, b = 0;
        if (!read_uint(i, &a)) {
            *err = "edge index is not an integer";
            return false;
        }
        skip(i);
        if (i >= s.size() || s[i] != ',') {
            *err = "edge entry must have exactly 2 indices";
            return false;
        }
        ++i;
        if (!read_uint(i, &b)) {
            *err = "edge index is not an integer";
            return false;
        }
        skip(i);
        if (i >= s.size() || s[i] != ']') {
            *err = "edge entry must have exactly 2 indices";
            return false;
        }
        ++i;
        edges->push_back((int32_t)a);
        edges->push_back((int32_t)b);
        skip(i);
        if (i < s.size() && s[i] == ',') ++i;
    }
    return true;
}

std::string file_stem(const std::string& path) {
    size_t slash = path.find_last_of('/');
    std::string base = slash == std::string::npos ? path : path.substr(slash + 1);
    size_t dot = base.find_last_of('.');
    if (dot != std::string::npos && dot > 0) base = base.substr(0, dot);
    return base.empty() ? "graph" : base;
}

}  // namespace

int main(int argc, char** argv) {
    using namespace rcli;
    std::string model = "ising", graph_path, outdir = "analysis/data";
    double t_min = 6.0, t_max = 6.7, j = 1.0;
    uint64_t R = 20, warmup = 5000, samples = 50000, ee = 10, seed = 42;
    int i = 1;
    while (i < argc) {
        const std::string f = argv[i];
        if (f == "--model") model = get_arg(argc, argv, i, "--model"), i += 2;
        else if (f == "--graph") graph_path = get_arg(argc, argv, i, "--graph"), i += 2;
        else if (f == "--outdir") outdir = get_arg(argc, argv, i, "--outdir"), i += 2;
        else if (f == "--tmin") t_min = parse_arg<double>(argc, argv, i, "--tmin"), i += 2;
        else if (f == "--tmax") t_max = parse_arg<double>(argc, argv, i, "--tmax"), i += 2;
        else if (f == "--replicas") R = parse_arg<uint64_t>(argc, argv, i, "--replicas"), i += 2;
        else if (f == "--warmup") warmup = parse_arg<uint64_t>(argc, argv, i, "--warmup"), i += 2;
        else if (f == "--samples") samples = parse_arg<uint64_t>(argc, argv, i, "--samples"), i += 2;
        else if (f == "--exchange-every")
            ee = parse_arg<uint64_t>(argc, argv, i, "--exchange-every"), i += 2;
        else if (f == "--seed") seed = parse_arg<uint64_t>(argc, argv, i, "--seed"), i += 2;
        else if (f == "--j") j = parse_arg<double>(argc, argv, i, "--j"), i += 2;
        else i += 1;
    }
    if (graph_path.empty()) die("Error: --graph <path.json> is required");
    if (t_min <= 0.0) die("Error: --tmin must be positive (got " + rust_f64(t_min) + ")");
    if (t_max <= 0.0) die("Error: --tmax must be positive (got " + rust_f64(t_max) + ")");
    if (t_min >= t_max)
        die("Error: --tmin (" + rust_f64(t_min) + ") must be less than --tmax (" + rust_f64(t_max) +
            ")");
    if (warmup == 0) die("Error: --warmup must be at least 1");
    if (samples == 0) die("Error: --samples must be at least 1");

    std::ifstream in(graph_path);
    if (!in) {
        die("Error: failed to read graph file " + graph_path + ": " + strerror(errno) +
            " (os error " + std::to_string(errno) + ")");
    }
    std::stringstream ss;
    ss << in.rdbuf();
    int n = 0;
    std::vector<int32_t> edges;
    std::string perr;
    if (!parse_graph(ss.str(), &n, &edges, &perr)) panic_expect("failed to parse graph JSON", perr);
    const std::string name = file_stem(graph_path);
    std::string err;
    if (!mkdirs(outdir, &err)) panic_expect("failed to create outdir", err);
    fprintf(stderr, "jfit: model=%s, graph=%s, N=%d, T=%s..%s, replicas=%llu, exchange_every=%llu\n",
            model.c_str(), name.c_str(), n, rust_f64(t_min).c_str(), rust_f64(t_max).c_str(),
            (unsigned long long)R, (unsigned long long)ee);
    if (model != "ising" && model != "xy" && model != "heisenberg")
        die("Error: --model must be ising, xy, or heisenberg");
    if (R == 0) die("Error: --replicas must be at least 1");
    if (R > 1024) die("Error: --replicas must be at most 1024");
    if (ee == 0) {
        fprintf(stderr, "thread 'main' panicked at src/bin/gpu_jfit.rs:257:12:\n"
                        "attempt to calculate the remainder with a divisor of zero\n");
        return 101;
    }

    // linspace_temperatures (parallel_tempering.rs:39-46)
    std::vector<double> temps(R);
    for (uint64_t t = 0; t < R; ++t)
        temps[t] = R == 1 ? t_min : t_min + (t_max - t_min) * (double)t / (double)(R - 1);
    const double nn = (double)n;
    std::vector<double> se(R, 0.0), se2(R, 0.0), sm(R, 0.0), sm2(R, 0.0), sm4(R, 0.0);
    std::vector<uint64_t> cnt(R, 0);
    auto add = [&](int t, double e_per, double m_per) {
        se[t] += e_per;
        se2[t] += e_per * e_per;
        sm[t] += m_per;
        sm2[t] += m_per * m_per;
        sm4[t] += (m_per * m_per) * (m_per * m_per);
        ++cnt[t];
    };
    const uint64_t chunk = 10000;
    const int every = (int)std::min<uint64_t>(ee, 1u << 30);
    std::vector<int32_t> rt;
    int64_t acc = 0;
    if (model == "ising") {
        isg_graph* h = nullptr;
        if (isg_graph_create(&h, n, edges.data(), (int)(edges.size() / 2), (int)R, seed) != ISG_OK)
            panic_expect("failed to create the graph replicas", isg_last_error());
        if (isg_graph_set_temperatures(h, temps.data(), j) != ISG_OK ||
            isg_graph_step(h, (int64_t)warmup) != ISG_OK || isg_graph_reset_sampling(h) != ISG_OK)
            panic_expect("GPU sweep failed", isg_last_error());
        std::vector<int64_t> rb, rm;
        for (uint64_t done = 0; done < samples;) {
            const uint64_t nsw = std::min(chunk, samples - done);
            rt.assign(nsw * R, 0);
            rb.assign(nsw * R, 0);
            rm.assign(nsw * R, 0);
            int64_t got = 0;
            if (isg_graph_pt_run(h, (int64_t)nsw, every, 1, rt.data(), rb.data(), rm.data(),
                                 (int64_t)nsw, &got) != ISG_OK)
                panic_expect("GPU sweep failed", isg_last_error());
            for (int64_t row = 0; row < got; ++row)
                for (uint64_t r = 0; r < R; ++r) {
                    const size_t o = (size_t)row * R + r;
                    add(rt[o], -(j * (double)rb[o]) / nn, std::fabs((double)rm[o] / nn));
                }
            done += nsw;
        }
        isg_graph_get_accepted(h, &acc);
        isg_graph_destroy(h);
    } else {
        const int nc = model == "heisenberg" ? 3 : 2;
        isg_cgraph* h = nullptr;
        if (isg_cgraph_create(&h, n, edges.data(), (int)(edges.size() / 2), (int)R, nc, seed) !=
            ISG_OK)
            panic_expect("failed to create the graph replicas", isg_last_error());
        if (isg_cgraph_set_temperatures(h, temps.data(), j) != ISG_OK ||
            isg_cgraph_step(h, (int64_t)warmup) != ISG_OK || isg_cgraph_reset_sampling(h) != ISG_OK)
            panic_expect("GPU sweep failed", isg_last_error());
        std::vector<double> re, rmv;
        for (uint64_t done = 0; done < samples;) {
            const uint64_t nsw = std::min(chunk, samples - done);
            rt.assign(nsw * R, 0);
            re.assign(nsw * R, 0.0);
            rmv.assign(nsw * R * nc, 0.0);
            int64_t got = 0;
            if (isg_cgraph_pt_run(h, (int64_t)nsw, every, 1, rt.data(), re.data(), rmv.data(),
                                  (int64_t)nsw, &got) != ISG_OK)
                panic_expect("GPU sweep failed", isg_last_error());
            for (int64_t row = 0; row < got; ++row)
                for (uint64_t r = 0; r < R; ++r) {
                    const size_t o = (size_t)row * R + r;
                    double m2 = 0.0;
                    for (int k = 0; k < nc; ++k) m2 += rmv[o * nc + k] * rmv[o * nc + k];
                    add(rt[o], re[o] / nn, std::sqrt(m2) / nn);
                }
            done += nsw;
        }
        isg_cgraph_get_accepted(h, &acc);
        isg_cgraph_destroy(h);
    }

    const std::string path = join_path(outdir, "gpu_jfit_" + model + "_" + name + ".csv");
    std::string csv = "T,E,E_err,M,M_err,M2,M2_err,M4,M4_err,Cv,Cv_err,chi,chi_err\n";
    char buf[256];
    for (uint64_t t = 0; t < R; ++t) {
        if (cnt[t] == 0) continue;
        const double s = (double)cnt[t];
        const double beta = 1.0 / temps[t];
        const double ae = se[t] / s, ae2 = se2[t] / s, am = sm[t] / s, am2 = sm2[t] / s,
                     am4 = sm4[t] / s;
        const double cv = beta * beta * (ae2 - ae * ae) * nn;
        const double chi = beta * (am2 - am * am) * nn;
        snprintf(buf, sizeof buf, "%.4f,%.6f,0.0,%.6f,0.0,%.6f,0.0,%.6f,0.0,%.6f,0.0,%.6f,0.0\n",
                 temps[t], ae, am, am2, am4, cv, chi);
        csv += buf;
        fprintf(stderr, "  T=%.3f M=%.4f\n", temps[t], am);
    }
    fprintf(stderr, "  PT exchanges accepted: %lld\n", (long long)acc);
    FILE* fp = fopen(path.c_str(), "w");
    if (!fp) panic_expect("failed to write CSV", strerror(errno));
    fwrite(csv.data(), 1, csv.size(), fp);
    fclose(fp);
    fprintf(stderr, "Wrote %s\n", path.c_str());
    return 0;
}
