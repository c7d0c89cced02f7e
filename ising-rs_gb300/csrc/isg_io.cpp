// isg_io.cpp — binary files of the PT runs: the per-sample timeseries and the
// device energy histograms, for the reweighting consumers
// (analysis/scripts/reweighting.py, analysis/scripts/analyze_gpu_fss.py).
//
// The reference writes the timeseries as text, one "temp_idx,E,M" row per
// sample with 8 decimals (src/bin/gpu_fss.rs:212-290), and plans a compact
// binary form (docs/plans/2026-03-08-gpu-acceleration-design.md:138).  These
// files keep every value exactly (FP64) in a fixed little-endian layout that
// include/isg.h documents; the text files stay the default of the drivers.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "isg.h"

namespace isg {
int fail(int code, const std::string& msg);
}

using isg::fail;

namespace {

void put_u32(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 0; i < 4; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}
void put_u64(std::vector<unsigned char>& b, uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}
void put_f64(std::vector<unsigned char>& b, double x) {
    uint64_t v;
    std::memcpy(&v, &x, 8);
    put_u64(b, v);
}

}  // namespace

struct isg_ts {
    FILE* f = nullptr;
    int n_temps = 0;
    int64_t records = 0;
};

extern "C" {

int isg_ts_open(isg_ts** out, const char* path, int model, int n, const double* temps,
                int n_temps) {
    if (!out || !path) return fail(ISG_ERR_ARG, "isg_ts_open: NULL argument");
    *out = nullptr;
    if (model < 0 || model > 2 || n < 1 || n_temps < 0 || (n_temps > 0 && !temps))
        return fail(ISG_ERR_ARG, "isg_ts_open: bad header values");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ISG_ERR_ARG, std::string("isg_ts_open: ") + path + ": " + std::strerror(errno));
    std::vector<unsigned char> b;
    const char magic[8] = {'I', 'S', 'G', 'T', 'S', 'E', 'R', '1'};
    b.insert(b.end(), magic, magic + 8);
    put_u32(b, (uint32_t)(32 + 8 * n_temps));
    put_u32(b, (uint32_t)model);
    put_u32(b, (uint32_t)n);
    put_u32(b, (uint32_t)n_temps);
    put_u64(b, 0);
    for (int t = 0; t < n_temps; ++t) put_f64(b, temps[t]);
    if (std::fwrite(b.data(), 1, b.size(), f) != b.size()) {
        std::fclose(f);
        return fail(ISG_ERR_ARG, "isg_ts_open: write failed");
    }
    isg_ts* h = new (std::nothrow) isg_ts();
    if (!h) {
        std::fclose(f);
        return fail(ISG_ERR_ARG, "isg_ts_open: out of host memory");
    }
    h->f = f;
    h->n_temps = n_temps;
    *out = h;
    return ISG_OK;
}

int isg_ts_append(isg_ts* h, const int32_t* temp_idx, const int32_t* replica, const double* e,
                  const double* m, int64_t count) {
    if (!h || !h->f || count < 0 || (count > 0 && (!temp_idx || !replica || !e || !m)))
        return fail(ISG_ERR_ARG, "isg_ts_append: bad argument");
    std::vector<unsigned char> b;
    b.reserve((size_t)count * 24);
    for (int64_t i = 0; i < count; ++i) {
        if (temp_idx[i] < 0 || temp_idx[i] >= h->n_temps)
            return fail(ISG_ERR_ARG, "isg_ts_append: temperature index out of range");
        put_u32(b, (uint32_t)temp_idx[i]);
        put_u32(b, (uint32_t)replica[i]);
        put_f64(b, e[i]);
        put_f64(b, m[i]);
    }
    if (!b.empty() && std::fwrite(b.data(), 1, b.size(), h->f) != b.size())
        return fail(ISG_ERR_ARG, "isg_ts_append: write failed");
    h->records += count;
    return ISG_OK;
}

int isg_ts_close(isg_ts* h) {
    if (!h) return ISG_OK;
    int rc = ISG_OK;
    if (h->f && std::fclose(h->f) != 0) rc = fail(ISG_ERR_ARG, "isg_ts_close: close failed");
    delete h;
    return rc;
}

int isg_hist_write(const char* path, int dim, int n, double J, const double* temps, int n_temps,
                   const int64_t* bond_lo, const int64_t* n_bins, const uint64_t* counters) {
    if (!path || dim < 2 || dim > 3 || n < 1 || n_temps < 0 ||
        (n_temps > 0 && (!temps || !bond_lo || !n_bins)))
        return fail(ISG_ERR_ARG, "isg_hist_write: bad argument");
    int64_t total = 0;
    for (int t = 0; t < n_temps; ++t) {
        if (n_bins[t] < 0) return fail(ISG_ERR_ARG, "isg_hist_write: negative bin count");
        total += n_bins[t];
    }
    if (total > 0 && !counters) return fail(ISG_ERR_ARG, "isg_hist_write: NULL counters");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ISG_ERR_ARG, std::string("isg_hist_write: ") + path + ": " + std::strerror(errno));
    std::vector<unsigned char> b;
    const char magic[8] = {'I', 'S', 'G', 'H', 'I', 'S', 'T', '1'};
    b.insert(b.end(), magic, magic + 8);
    put_u32(b, (uint32_t)(32 + 8 * n_temps));
    put_u32(b, (uint32_t)dim);
    put_u32(b, (uint32_t)n);
    put_u32(b, (uint32_t)n_temps);
    put_f64(b, J);
    for (int t = 0; t < n_temps; ++t) put_f64(b, temps[t]);
    const uint64_t* c = counters;
    for (int t = 0; t < n_temps; ++t) {
        put_u64(b, (uint64_t)bond_lo[t]);
        put_u64(b, (uint64_t)n_bins[t]);
        for (int64_t i = 0; i < 4 * n_bins[t]; ++i) put_u64(b, c[i]);
        c += 4 * n_bins[t];
    }
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    if (std::fclose(f) != 0 || !ok) return fail(ISG_ERR_ARG, "isg_hist_write: write failed");
    return ISG_OK;
}

}  // extern "C"
