// mc_report.cpp -- mc_report(): the output.h5 layout written as JSON.
//
// Simulator::report (src/simulator/report.cpp:9-50) and Estimator::report
// (src/Estimator.cpp:368-422) write, with the HDF5 C++ API:
//   /summary/{Ncycle, Nsample, Npassive, Ntrack, mode}
//   /summary/survival_roulette/{wr, ws}
//   /<estimator> with attribute "indexing" = "[filter1][filter2]...",
//       one dataset per filter (its grid, attribute "unit"),
//       /<estimator>/<score>/{mean, uncertainty} shaped by the filter sizes.
// HDF5 is not available here, so the same tree is written as nested JSON
// objects, datasets as (nested) arrays in row-major order.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "mc_engine.h"
#include "mc_handle.h"
#include "mcgpu.h"

using namespace mc;


namespace {

const char *filter_name(int k)
{
    switch (k) {
    case F_SURFACE: return "surface";
    case F_CELL: return "cell";
    case F_ENERGY: return "energy";
    case F_TIME: return "time";
    default: return "group";
    }
}

const char *filter_unit(int k)
{
    switch (k) {
    case F_SURFACE: case F_CELL: return "id#";
    case F_ENERGY: return "eV";
    case F_TIME: return "s";
    default: return "group#";
    }
}

std::string num(double v)
{
    if (std::isnan(v)) return "NaN";
    if (std::isinf(v)) return v > 0 ? "Infinity" : "-Infinity";
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    return b;
}

std::string quote(const std::string &s)
{
    std::string o = "\"";
    for (char c : s) {
        if (c == '"' || c == '\\') o += '\\';
        o += c;
    }
    return o + "\"";
}

// row-major nested array of vals with the given dims
void nested(std::string &o, const double *vals, const std::vector<int> &dims, size_t d)
{
    if (dims.empty()) { o += num(vals[0]); return; }
    size_t stride = 1;
    for (size_t k = d + 1; k < dims.size(); ++k) stride *= (size_t)dims[k];
    o += "[";
    for (int i = 0; i < dims[d]; ++i) {
        if (i) o += ", ";
        if (d + 1 == dims.size()) o += num(vals[i]);
        else nested(o, vals + (size_t)i * stride, dims, d + 1);
    }
    o += "]";
}

}  // namespace

extern "C" mc_status mc_report(const mc_problem *p, const char *path)
{
    if (!p || !path) return MC_ERR_ARG;
    const Tables &t = p->t;
    std::vector<double> sum, sq;
    std::string err;
    mc_status st = read_sums(p->dev, sum, sq, err);
    if (st != MC_OK) { const_cast<mc_problem *>(p)->err = err; return st; }
    const double N = (double)p->dev.histories;
    std::string o = "{\n \"summary\": {\"Ncycle\": 1, \"Nsample\": " + std::to_string(p->dev.histories) +
                    ", \"Npassive\": 0, \"Ntrack\": " + std::to_string(p->dev.ntrack) +
                    ", \"mode\": \"fixed source\", \"survival_roulette\": {\"wr\": " + num(t.wr) +
                    ", \"ws\": " + num(t.ws) + "}}";
    for (int e = 0; e < t.n_est(); ++e) {
        const int f0 = t.est_filt_off[e], f1 = t.est_filt_off[e + 1];
        std::string indexing;
        std::vector<int> dims;
        for (int f = f0; f < f1; ++f) {
            indexing += std::string("[") + filter_name(t.filt_kind[f]) + "]";
            dims.push_back(t.filt_size[f]);
        }
        o += ",\n " + quote(t.est_names[e]) + ": {\"indexing\": " + quote(indexing);
        for (int f = f0; f < f1; ++f) {
            o += ", " + quote(filter_name(t.filt_kind[f])) + ": {\"unit\": " + quote(filter_unit(t.filt_kind[f])) +
                 ", \"grid\": [";
            for (int g = 0; g < t.filt_grid_len[f]; ++g) {
                if (g) o += ", ";
                o += num(t.filt_grid[t.filt_grid_off[f] + g]);
            }
            o += "]}";
        }
        size_t per_score = 1;
        for (int dsz : dims) per_score *= (size_t)dsz;
        const int s0 = t.est_score_off[e], s1 = t.est_score_off[e + 1];
        for (int s = s0; s < s1; ++s) {
            std::vector<double> mean(per_score), unc(per_score);
            const size_t base = (size_t)t.est_bin_off[e] + (size_t)(s - s0) * per_score;
            for (size_t j = 0; j < per_score; ++j) {
                const double m = sum[base + j] / N;
                mean[j] = m;
                unc[j] = std::sqrt((sq[base + j] / N - m * m) / (N - 1.0));
            }
            o += ", " + quote(t.est_score_names[e][s - s0]) + ": {\"mean\": ";
            nested(o, mean.data(), dims, 0);
            o += ", \"uncertainty\": ";
            nested(o, unc.data(), dims, 0);
            o += "}";
        }
        o += "}";
    }
    o += "\n}\n";
    FILE *f = std::fopen(path, "w");
    if (!f) { const_cast<mc_problem *>(p)->err = std::string("cannot write ") + path; return MC_ERR_ARG; }
    std::fwrite(o.data(), 1, o.size(), f);
    std::fclose(f);
    return MC_OK;
}
