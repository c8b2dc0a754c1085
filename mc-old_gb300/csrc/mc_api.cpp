// mc_api.cpp -- the C ABI of include/mcgpu.h.
//
// Host side of the library: owns the problem tables (host and device), the
// per-handle CUDA stream, the accumulated tallies and the scratch buffers of
// the transport engines, and turns every failure into a status code.
#include "mcgpu.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <string>
#include <vector>

#include "mc_device.h"
#include "mc_engine.h"
#include "mc_handle.h"
#include "mc_problem.h"

using namespace mc;


namespace {

mc_status fail(mc_problem *p, mc_status s, const std::string &msg)
{
    if (p) p->err = msg;
    return s;
}

}  // namespace

extern "C" {

const char *mc_status_string(mc_status s)
{
    switch (s) {
    case MC_OK: return "MC_OK";
    case MC_ERR_INPUT: return "MC_ERR_INPUT";
    case MC_ERR_CUDA: return "MC_ERR_CUDA";
    case MC_ERR_OVERFLOW: return "MC_ERR_OVERFLOW";
    case MC_ERR_LOST: return "MC_ERR_LOST";
    case MC_ERR_TIMEOUT: return "MC_ERR_TIMEOUT";
    case MC_ERR_NAN: return "MC_ERR_NAN";
    case MC_ERR_NOMEM: return "MC_ERR_NOMEM";
    case MC_ERR_ARG: return "MC_ERR_ARG";
    }
    return "MC_ERR_UNKNOWN";
}

const char *mc_last_error(const mc_problem *p)
{
    if (!p) return "null problem handle";
    return p->err.c_str();
}

mc_status mc_problem_load_xml(const char *io_dir, const char *xs_dir, mc_problem **out)
{
    if (!io_dir || !out) return MC_ERR_ARG;
    *out = nullptr;
    mc_problem *p = new (std::nothrow) mc_problem();
    if (!p) return MC_ERR_NOMEM;
    std::string err;
    const std::string xs = xs_dir ? std::string(xs_dir) : std::string("./xs_library");
    if (!load_problem(io_dir, xs, p->t, err)) {
        // keep the handle so the caller can read the message, as the
        // reference prints its own before exiting
        p->err = err;
        *out = p;
        return MC_ERR_INPUT;
    }
    mc_status s = device_problem_init(p->t, p->dev, err);
    if (s != MC_OK) {
        p->err = err;
        *out = p;
        return s;
    }
    *out = p;
    return MC_OK;
}

mc_status mc_problem_upload(mc_problem *p)
{
    if (!p) return MC_ERR_ARG;
    if (!p->dev.ready) return fail(p, MC_ERR_ARG, "problem was not loaded");
    std::string err;
    mc_status s = upload_tables(p->dev, err);
    if (s == MC_OK) s = event_tables_upload(p->dev, err);
    if (s != MC_OK) p->err = err;
    return s;
}

mc_status mc_problem_table_bytes(const mc_problem *p, uint64_t *bytes)
{
    if (!p || !bytes) return MC_ERR_ARG;
    *bytes = (uint64_t)(p->dev.blob_bytes + event_table_bytes(p->dev));
    return MC_OK;
}

mc_status mc_problem_free(mc_problem *p)
{
    if (!p) return MC_ERR_ARG;
    device_problem_free(p->dev);
    delete p;
    return MC_OK;
}

mc_status mc_run(mc_problem *p, uint64_t first, uint64_t n, uint64_t seed, mc_mode mode, const mc_tune *tune)
{
    if (!p) return MC_ERR_ARG;
    if (!p->dev.ready) return fail(p, MC_ERR_ARG, "problem was not loaded");
    if (mode != MC_FP64_REPLAY && mode != MC_FP64_PLAIN && mode != MC_MIXED_EVENT)
        return fail(p, MC_ERR_ARG, "unknown mode");
    std::string err;
    mc_status s = run_histories(p->t, p->dev, first, n, seed, mode, tune, err);
    if (s != MC_OK) p->err = err;
    return s;
}

mc_status mc_reset_tallies(mc_problem *p)
{
    if (!p) return MC_ERR_ARG;
    std::string err;
    mc_status s = reset_tallies(p->dev, err);
    if (s != MC_OK) p->err = err;
    return s;
}

// A problem's fingerprint for saved states: FNV-1a over the packed device
// tables (geometry, materials, cross sections, estimators, sources).
static uint64_t table_fingerprint(const DeviceProblem &d)
{
    uint64_t h = 0xCBF29CE484222325ULL;
    const unsigned char *b = static_cast<const unsigned char *>(d.h_blob);
    for (size_t i = 0; i < d.blob_bytes; ++i) h = (h ^ b[i]) * 0x100000001B3ULL;
    return h;
}

static const char kStateMagic[8] = {'M', 'C', 'G', 'P', 'U', 'S', 'T', '1'};

mc_status mc_state_save(const mc_problem *p, const char *path)
{
    if (!p || !path) return MC_ERR_ARG;
    std::vector<double> s, q;
    std::string err;
    mc_status st = read_sums(p->dev, s, q, err);
    if (st != MC_OK) { const_cast<mc_problem *>(p)->err = err; return st; }
    const uint64_t head[4] = {(uint64_t)s.size(), p->dev.histories, p->dev.ntrack, table_fingerprint(p->dev)};
    FILE *f = std::fopen(path, "wb");
    if (!f) { const_cast<mc_problem *>(p)->err = std::string("cannot write ") + path; return MC_ERR_ARG; }
    const bool ok = std::fwrite(kStateMagic, 1, 8, f) == 8 && std::fwrite(head, 8, 4, f) == 4 &&
                    std::fwrite(s.data(), 8, s.size(), f) == s.size() &&
                    std::fwrite(q.data(), 8, q.size(), f) == q.size();
    if (std::fclose(f) != 0 || !ok) {
        const_cast<mc_problem *>(p)->err = std::string("cannot write ") + path;
        return MC_ERR_ARG;
    }
    return MC_OK;
}

mc_status mc_state_load(mc_problem *p, const char *path)
{
    if (!p || !path) return MC_ERR_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(p, MC_ERR_INPUT, std::string("cannot read ") + path);
    char magic[8];
    uint64_t head[4];
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kStateMagic, 8) == 0 &&
              std::fread(head, 8, 4, f) == 4;
    const size_t nb = (size_t)std::max<long long>(p->dev.dt.n_bins, 1);
    std::vector<double> s, q;
    if (ok && head[0] == nb && head[3] == table_fingerprint(p->dev)) {
        s.resize(nb);
        q.resize(nb);
        ok = std::fread(s.data(), 8, nb, f) == nb && std::fread(q.data(), 8, nb, f) == nb;
    } else {
        ok = false;
    }
    std::fclose(f);
    if (!ok) return fail(p, MC_ERR_INPUT, std::string(path) + " is not a saved state of this problem");
    DeviceProblem &d = p->dev;
    cudaError_t e;
    if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess ||
        (e = cudaMemcpy(d.d_sum, s.data(), nb * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(d.d_sq, q.data(), nb * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(p, MC_ERR_CUDA, cuda_msg(e, "load tallies"));
    d.histories = head[1];
    d.ntrack = head[2];
    d.exact_valid = false;   // the saved state holds the FP64 sums only
    return MC_OK;
}

mc_status mc_exact_sums_read(const mc_problem *p, int64_t *limbs, uint64_t cap)
{
    if (!p || !limbs) return MC_ERR_ARG;
    const DeviceProblem &d = p->dev;
    const size_t nb = (size_t)std::max<long long>(d.dt.n_bins, 0);
    const size_t need = nb * 2 * kExactLimbs;
    if (cap < need)
        return fail(const_cast<mc_problem *>(p), MC_ERR_ARG,
                    "mc_exact_sums_read: the buffer holds " + std::to_string(cap) + " limbs, " +
                        std::to_string(need) + " are needed (n_bins x 2 x MC_EXACT_LIMBS)");
    if (!d.exact_valid)
        return fail(const_cast<mc_problem *>(p), MC_ERR_ARG,
                    "mc_exact_sums_read: a run since the last reset was not an FP64 run (or the tallies "
                    "were loaded from a saved state), so the exact sums do not cover them");
    if (need == 0) return MC_OK;
    cudaError_t e;
    if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess ||
        (e = cudaMemcpy(limbs, d.d_exact, need * sizeof(int64_t), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail(const_cast<mc_problem *>(p), MC_ERR_CUDA, cuda_msg(e, "read exact sums"));
    return MC_OK;
}

mc_status mc_exact_round(const int64_t *limbs, uint64_t n_values, double *out)
{
    if ((!limbs || !out) && n_values) return MC_ERR_ARG;
    for (uint64_t i = 0; i < n_values; ++i) out[i] = exact_round(limbs + i * kExactLimbs);
    return MC_OK;
}

mc_status mc_tally_count(const mc_problem *p, uint32_t *n)
{
    if (!p || !n) return MC_ERR_ARG;
    *n = (uint32_t)p->t.n_est();
    return MC_OK;
}

mc_status mc_tally_size(const mc_problem *p, uint32_t est, uint64_t *n)
{
    if (!p || !n || est >= (uint32_t)p->t.n_est()) return MC_ERR_ARG;
    *n = (uint64_t)(p->t.est_bin_off[est + 1] - p->t.est_bin_off[est]);
    return MC_OK;
}

mc_status mc_estimator_name(const mc_problem *p, uint32_t est, char *buf, size_t cap)
{
    if (!p || !buf || cap == 0 || est >= (uint32_t)p->t.n_est()) return MC_ERR_ARG;
    std::snprintf(buf, cap, "%s", p->t.est_names[est].c_str());
    return MC_OK;
}

mc_status mc_tally_read(const mc_problem *p, uint32_t est, double *mean, double *sigma, double *sum,
                        double *sumsq, uint64_t cap)
{
    if (!p || est >= (uint32_t)p->t.n_est()) return MC_ERR_ARG;
    const int64_t b0 = p->t.est_bin_off[est], b1 = p->t.est_bin_off[est + 1];
    const uint64_t nb = (uint64_t)(b1 - b0);
    if (cap < nb && (mean || sigma || sum || sumsq)) return MC_ERR_ARG;
    std::vector<double> s, q;
    std::string err;
    mc_status st = read_sums(p->dev, s, q, err);
    if (st != MC_OK) { const_cast<mc_problem *>(p)->err = err; return st; }
    // Estimator::end_cycle / end_simulation for one active cycle
    // (Estimator.cpp:347-367) with N = histories folded so far
    const double N = (double)p->dev.histories;
    for (uint64_t j = 0; j < nb; ++j) {
        const double sv = s[b0 + j], qv = q[b0 + j];
        const double m = sv / N;
        const double us = (qv / N - m * m) / (N - 1.0);
        if (mean) mean[j] = (0.0 + m) / 1.0;
        if (sigma) sigma[j] = std::sqrt(0.0 + us) / 1.0;
        if (sum) sum[j] = sv;
        if (sumsq) sumsq[j] = qv;
    }
    return MC_OK;
}

mc_status mc_counters_read(const mc_problem *p, mc_counters *out)
{
    if (!p || !out) return MC_ERR_ARG;
    *out = p->dev.last;
    return MC_OK;
}

mc_status mc_digests_read(const mc_problem *p, uint64_t *out, uint64_t cap)
{
    if (!p || !out) return MC_ERR_ARG;
    if (cap < p->dev.digests.size()) return MC_ERR_ARG;
    std::memcpy(out, p->dev.digests.data(), p->dev.digests.size() * sizeof(uint64_t));
    return MC_OK;
}

mc_status mc_nsample(const mc_problem *p, uint64_t *n)
{
    if (!p || !n) return MC_ERR_ARG;
    *n = p->t.nsample;
    return MC_OK;
}

mc_status mc_histories_run(const mc_problem *p, uint64_t *n)
{
    if (!p || !n) return MC_ERR_ARG;
    *n = p->dev.histories;
    return MC_OK;
}

}  // extern "C"
