// mc_lr.cpp -- forward / backward pair for tally derivatives.
//
// The reference has no derivative capability.  For one-group (multigroup,
// G = 1) problems the parameters are every material's (Sigma_s, Sigma_a).
// mc_forward runs the FP64 replay transport with those values; mc_backward
// runs the likelihood-ratio kernel (k_history_fp64<true, true>), which
// carries each particle's score-function weights S_k = d ln(w x path
// probability)/d param_k along the history and adds v S_k (plus the direct
// dependence of a Sigma-weighted score) for every tally contribution v.  The
// per-history derivative totals are folded like the tallies themselves, so
// every derivative comes with its standard error.  Both calls use the
// problem's seed keying, so forward runs at perturbed parameters with the
// same seed and history range are common-random-number finite differences.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mc_device.h"
#include "mc_engine.h"
#include "mc_handle.h"
#include "mcgpu.h"

using namespace mc;

namespace {

struct LrScratch {
    DevBuf tab, rows, stack, lrstack, sums, misc;
};

LrScratch &scratch_of(mc_problem *p)
{
    // one scratch set per handle, kept next to the handle's other buffers
    static_assert(sizeof(LrScratch) > 0, "");
    if (!p->dev.lr) p->dev.lr = new LrScratch();
    return *static_cast<LrScratch *>(p->dev.lr);
}

mc_status check_one_group(mc_problem *p, const double *params)
{
    if (!p || !params) return MC_ERR_ARG;
    if (!p->dev.ready) { p->err = "problem was not loaded"; return MC_ERR_ARG; }
    if (p->t.mg_groups != 1) {
        p->err = "forward/backward need a one-group multigroup problem (<multigroup groups=\"1\"/>)";
        return MC_ERR_ARG;
    }
    if (p->t.comb_teeth > 0) { p->err = "forward/backward do not support the particle comb"; return MC_ERR_ARG; }
    if (2 * p->t.n_mat() > kMaxLrParams) { p->err = "forward/backward support at most 32 materials"; return MC_ERR_ARG; }
    for (int i = 0; i < 2 * p->t.n_mat(); ++i)
        if (!(params[i] >= 0.0) || !std::isfinite(params[i])) { p->err = "cross sections must be finite and >= 0"; return MC_ERR_ARG; }
    return MC_OK;
}

// Runs histories [first, first + n) in FP64 replay with the materials'
// one-group cross sections replaced by params; with_lr adds the derivative
// columns.  Leaves per-column sums / sums of squares in S.sums.
mc_status run_params(mc_problem *p, const double *params, uint64_t n, uint64_t seed, bool with_lr,
                     std::vector<double> &sum, std::vector<double> &sq)
{
    DeviceProblem &d = p->dev;
    LrScratch &S = scratch_of(p);
    const int nm = p->t.n_mat();
    const int K = with_lr ? 2 * nm : 0;
    const int Kc = with_lr ? 3 * nm : 0;   // (Sigma_s, Sigma_a) pairs, then rho d/drho per material
    const long long nb = std::max<long long>(d.dt.n_bins, 1);
    const long long row = nb * (1 + Kc);
    // one-group tables with the new values, built the way the reader builds
    // them (capture = total - scatter row sum)
    std::vector<double> tot(nm), sca(nm), stot(nm), cap(nm);
    for (int m = 0; m < nm; ++m) {
        const double ss = params[2 * m], sa = params[2 * m + 1];
        tot[m] = ss + sa;
        sca[m] = ss;
        stot[m] = 0.0 + ss;
        cap[m] = tot[m] - stot[m];
    }
    const size_t tb = 4 * (size_t)nm * sizeof(double) + 4 * 256;
    if (!devbuf_reserve(S.tab, tb)) { p->err = "cannot allocate parameter tables"; return MC_ERR_NOMEM; }
    char *tp = static_cast<char *>(S.tab.ptr);
    DevTables T = d.dt;
    const size_t step = ((size_t)nm * sizeof(double) + 255) & ~(size_t)255;
    cudaMemcpyAsync(tp, tot.data(), nm * sizeof(double), cudaMemcpyHostToDevice, d.stream);
    cudaMemcpyAsync(tp + step, sca.data(), nm * sizeof(double), cudaMemcpyHostToDevice, d.stream);
    cudaMemcpyAsync(tp + 2 * step, stot.data(), nm * sizeof(double), cudaMemcpyHostToDevice, d.stream);
    cudaMemcpyAsync(tp + 3 * step, cap.data(), nm * sizeof(double), cudaMemcpyHostToDevice, d.stream);
    T.mg_total = reinterpret_cast<const double *>(tp);
    T.mg_scatter = reinterpret_cast<const double *>(tp + step);
    T.mg_scat_tot = reinterpret_cast<const double *>(tp + 2 * step);
    T.mg_capture = reinterpret_cast<const double *>(tp + 3 * step);

    const int block = 128;
    const uint32_t depth = 32;
    const int grid = std::max(1, history_fp64_max_threads(true, block) / block);
    const uint64_t threads = (uint64_t)grid * block;
    uint64_t chunk = (uint64_t)((1ull << 30) / (row * sizeof(double)));
    chunk = std::max<uint64_t>(1, std::min<uint64_t>({chunk, 1u << 22, n}));
    if (!devbuf_reserve(S.rows, (size_t)chunk * row * sizeof(double)) ||
        !devbuf_reserve(S.stack, (size_t)threads * depth * fp64_particle_bytes()) ||
        (K && !devbuf_reserve(S.lrstack, (size_t)threads * depth * K * sizeof(double))) ||
        !devbuf_reserve(S.sums, 2 * (size_t)row * sizeof(double)) ||
        !devbuf_reserve(S.misc, 256 + kNumCounters * sizeof(unsigned long long))) {
        p->err = "cannot allocate derivative scratch";
        return MC_ERR_NOMEM;
    }
    double *dsum = static_cast<double *>(S.sums.ptr);
    double *dsq = dsum + row;
    char *misc = static_cast<char *>(S.misc.ptr);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(misc);
    int *status = reinterpret_cast<int *>(misc + kNumCounters * 8);
    unsigned int *next = reinterpret_cast<unsigned int *>(misc + kNumCounters * 8 + 16);
    cudaMemsetAsync(dsum, 0, 2 * (size_t)row * sizeof(double), d.stream);
    cudaMemsetAsync(misc, 0, 256 + kNumCounters * sizeof(unsigned long long), d.stream);
    cudaError_t e;
    for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
        const uint32_t cn = (uint32_t)std::min<uint64_t>(chunk, n - c0);
        HistoryArgs A;
        A.first = c0;
        A.n = cn;
        A.seed = seed;
        A.hist = static_cast<double *>(S.rows.ptr);
        A.stack = S.stack.ptr;
        A.stack_depth = depth;
        A.counters = cnt;
        A.digest = nullptr;
        A.status = status;
        A.next = next;
        A.n_params = K;
        A.n_cols = Kc;
        A.lr_stack = K ? static_cast<double *>(S.lrstack.ptr) : nullptr;
        if ((e = cudaMemsetAsync(next, 0, sizeof(unsigned int), d.stream)) != cudaSuccess ||
            (e = launch_history_fp64(T, A, true, grid, block, d.stream)) != cudaSuccess ||
            (e = launch_fold(A.hist, cn, row, dsum, dsq, true, d.stream)) != cudaSuccess) {
            p->err = cuda_msg(e, "derivative kernels");
            return MC_ERR_CUDA;
        }
    }
    int hs = 0;
    sum.assign(row, 0.0);
    sq.assign(row, 0.0);
    if ((e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sum.data(), dsum, row * sizeof(double), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sq.data(), dsq, row * sizeof(double), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        p->err = cuda_msg(e, "derivative kernels");
        return MC_ERR_CUDA;
    }
    if (hs != DS_OK) {
        p->err = "device error status in the derivative run";
        return status_from_device(hs);
    }
    return MC_OK;
}

void stats(const std::vector<double> &sum, const std::vector<double> &sq, size_t from, size_t count, double N,
           double *mean, double *sigma)
{
    for (size_t j = 0; j < count; ++j) {
        const double m = sum[from + j] / N;
        if (mean) mean[j] = m;
        if (sigma) sigma[j] = std::sqrt(std::max(0.0, (sq[from + j] / N - m * m) / (N - 1.0)));
    }
}

}  // namespace

void mc::lr_scratch_free(void *lr)
{
    if (!lr) return;
    LrScratch *S = static_cast<LrScratch *>(lr);
    devbuf_free(S->tab); devbuf_free(S->rows); devbuf_free(S->stack);
    devbuf_free(S->lrstack); devbuf_free(S->sums); devbuf_free(S->misc);
    delete S;
}

extern "C" {

mc_status mc_lr_params(const mc_problem *p, double *params, uint32_t cap)
{
    if (!p || !params) return MC_ERR_ARG;
    if (p->t.mg_groups != 1) { const_cast<mc_problem *>(p)->err = "not a one-group multigroup problem"; return MC_ERR_ARG; }
    const int nm = p->t.n_mat();
    if (cap < (uint32_t)(2 * nm)) return MC_ERR_ARG;
    for (int m = 0; m < nm; ++m) {
        params[2 * m] = p->t.mg_scat_tot[m];
        params[2 * m + 1] = p->t.mg_capture[m];
    }
    return MC_OK;
}

mc_status mc_forward(mc_problem *p, const double *params, uint64_t n, uint64_t seed, double *tally_out,
                     double *sigma_out)
{
    mc_status st = check_one_group(p, params);
    if (st != MC_OK) return st;
    if (n < 2) { p->err = "need at least two histories"; return MC_ERR_ARG; }
    std::vector<double> sum, sq;
    if ((st = run_params(p, params, n, seed, false, sum, sq)) != MC_OK) return st;
    stats(sum, sq, 0, (size_t)p->t.n_bins(), (double)n, tally_out, sigma_out);
    return MC_OK;
}

mc_status mc_backward_density(mc_problem *p, const double *params, uint64_t n, uint64_t seed, double *dtally,
                              double *sigma, double *drho, double *drho_sigma)
{
    mc_status st = check_one_group(p, params);
    if (st != MC_OK) return st;
    if (!dtally && !drho) return MC_ERR_ARG;
    if (n < 2) { p->err = "need at least two histories"; return MC_ERR_ARG; }
    std::vector<double> sum, sq;
    if ((st = run_params(p, params, n, seed, true, sum, sq)) != MC_OK) return st;
    const size_t nb = (size_t)p->t.n_bins();
    const size_t nm = (size_t)p->t.n_mat();
    const size_t K = 2 * nm, Kc = 3 * nm;
    const size_t base = std::max<size_t>(nb, 1);
    std::vector<double> m(Kc), s(Kc);
    for (size_t b = 0; b < nb; ++b) {
        stats(sum, sq, base + b * Kc, Kc, (double)n, m.data(), s.data());
        for (size_t k = 0; k < K; ++k) {
            if (dtally) dtally[b * K + k] = m[k];
            if (sigma) sigma[b * K + k] = s[k];
        }
        for (size_t k = 0; k < nm; ++k) {
            if (drho) drho[b * nm + k] = m[K + k];
            if (drho_sigma) drho_sigma[b * nm + k] = s[K + k];
        }
    }
    return MC_OK;
}

mc_status mc_backward(mc_problem *p, const double *params, uint64_t n, uint64_t seed, double *dtally,
                      double *sigma)
{
    if (!dtally) return MC_ERR_ARG;
    return mc_backward_density(p, params, n, seed, dtally, sigma, nullptr, nullptr);
}

}  // extern "C"
