// mc_engine.cpp -- device tables, tally accumulation and the FP64 history
// engine driver (see mc_engine.h).
#include "mc_engine.h"

#include <algorithm>
#include <cstring>

namespace mc {

std::string cuda_msg(cudaError_t e, const char *what)
{
    return std::string(what) + ": " + cudaGetErrorString(e);
}

mc_status status_from_device(int ds)
{
    switch (ds) {
    case DS_OK: return MC_OK;
    case DS_OVERFLOW: return MC_ERR_OVERFLOW;
    case DS_LOST: return MC_ERR_LOST;
    case DS_TIMEOUT: return MC_ERR_TIMEOUT;
    case DS_NAN: return MC_ERR_NAN;
    default: return MC_ERR_CUDA;
    }
}

const char *device_status_text(int ds)
{
    switch (ds) {
    case DS_LOST: return "a particle was lost (no cell contains it)";
    case DS_OVERFLOW: return "split stack or filter buffer overflow";
    case DS_TIMEOUT:
        return "a particle exceeded the event limit, a history its particle limit, or the free-gas loop its "
               "candidate limit";
    case DS_NAN: return "a non-finite track length, energy or weight";
    default: return "device error status";
    }
}

bool devbuf_reserve(DevBuf &buf, size_t bytes)
{
    if (bytes <= buf.bytes && buf.ptr) return true;
    if (buf.ptr) cudaFree(buf.ptr);
    buf.ptr = nullptr;
    buf.bytes = 0;
    if (bytes == 0) bytes = 256;
    if (cudaMalloc(&buf.ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        buf.ptr = nullptr;
        return false;
    }
    buf.bytes = bytes;
    return true;
}

void devbuf_free(DevBuf &buf)
{
    if (buf.ptr) cudaFree(buf.ptr);
    buf.ptr = nullptr;
    buf.bytes = 0;
}

namespace {

// Packs host vectors into one staging buffer (256-byte aligned sections) and
// records where each lands so the device pointers can be patched in.
struct Packer {
    std::vector<char> buf;
    std::vector<std::pair<const void **, size_t>> fix;

    template <class T>
    void add(const std::vector<T> &v, const T **slot)
    {
        size_t off = (buf.size() + 255) & ~(size_t)255;
        buf.resize(off + std::max<size_t>(v.size() * sizeof(T), 8), 0);
        if (!v.empty()) std::memcpy(buf.data() + off, v.data(), v.size() * sizeof(T));
        fix.emplace_back(reinterpret_cast<const void **>(slot), off);
    }
};

}  // namespace

mc_status device_problem_init(const Tables &t, DeviceProblem &d, std::string &err)
{
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        err = "no CUDA device available (the library has no CPU fallback)";
        return MC_ERR_CUDA;
    }
    cudaGetDevice(&d.device);
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, d.device);
    if ((e = cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking)) != cudaSuccess) {
        err = cuda_msg(e, "cudaStreamCreate");
        return MC_ERR_CUDA;
    }
    for (auto &ev : d.ev) cudaEventCreate(&ev);

    DevTables &T = d.dt;
    T.n_surf = t.n_surf(); T.n_cell = t.n_cell(); T.n_mat = t.n_mat(); T.n_nuc = t.n_nuc();
    T.mg_groups = t.mg_groups; T.n_est = t.n_est(); T.n_src = t.n_src();
    T.n_bins = t.n_bins();
    T.wr = t.wr; T.ws = t.ws;
    T.comb_bank_max = t.comb_bank_max; T.comb_teeth = t.comb_teeth;
    Packer P;
    P.add(t.surf_type, &T.surf_type); P.add(t.surf_bc, &T.surf_bc); P.add(t.surf_coef, &T.surf_coef);
    P.add(t.cell_imp, &T.cell_imp); P.add(t.cell_mat, &T.cell_mat); P.add(t.cell_surf_off, &T.cell_surf_off);
    P.add(t.cell_surf, &T.cell_surf); P.add(t.cell_sense, &T.cell_sense);
    P.add(t.cell_tl_off, &T.cell_tl_off); P.add(t.cell_tl, &T.cell_tl);
    P.add(t.cell_c_off, &T.cell_c_off); P.add(t.cell_c, &T.cell_c);
    P.add(t.surf_est_off, &T.surf_est_off); P.add(t.surf_est, &T.surf_est);
    P.add(t.mat_off, &T.mat_off); P.add(t.mat_nuc, &T.mat_nuc); P.add(t.mat_dens, &T.mat_dens);
    P.add(t.nuc_kind, &T.nuc_kind); P.add(t.nuc_len, &T.nuc_len); P.add(t.nuc_A, &T.nuc_A);
    P.add(t.nuc_const, &T.nuc_const);
    std::vector<long long> nuc_off(t.nuc_off.begin(), t.nuc_off.end());
    P.add(nuc_off, &T.nuc_off);
    P.add(t.xs_E, &T.xs_E); P.add(t.xs_S, &T.xs_S); P.add(t.xs_C, &T.xs_C); P.add(t.xs_T, &T.xs_T);
    P.add(t.mg_total, &T.mg_total); P.add(t.mg_scatter, &T.mg_scatter);
    P.add(t.mg_scat_tot, &T.mg_scat_tot); P.add(t.mg_capture, &T.mg_capture);
    P.add(t.est_score_off, &T.est_score_off); P.add(t.score_kind, &T.score_kind);
    P.add(t.score_kernel, &T.score_kernel); P.add(t.est_filt_off, &T.est_filt_off);
    P.add(t.filt_kind, &T.filt_kind); P.add(t.filt_size, &T.filt_size); P.add(t.filt_grid_len, &T.filt_grid_len);
    std::vector<long long> fgo(t.filt_grid_off.begin(), t.filt_grid_off.end());
    P.add(fgo, &T.filt_grid_off);
    P.add(t.filt_grid, &T.filt_grid); P.add(t.est_factor, &T.est_factor);
    P.add(t.est_factor_off, &T.est_factor_off);
    std::vector<long long> ebo(t.est_bin_off.begin(), t.est_bin_off.end());
    P.add(ebo, &T.est_bin_off);
    P.add(t.src_pos, &T.src_pos); P.add(t.src_dir_par, &T.src_dir_par); P.add(t.src_e_par, &T.src_e_par);
    P.add(t.src_cdf, &T.src_cdf); P.add(t.src_cell, &T.src_cell); P.add(t.src_dir_kind, &T.src_dir_kind);
    P.add(t.src_e_kind, &T.src_e_kind); P.add(t.src_group, &T.src_group);

    d.blob_bytes = P.buf.size();
    if ((e = cudaMalloc(&d.blob, d.blob_bytes)) != cudaSuccess) { err = cuda_msg(e, "cudaMalloc(tables)"); return MC_ERR_NOMEM; }
    if ((e = cudaHostAlloc(&d.h_blob, d.blob_bytes, cudaHostAllocDefault)) != cudaSuccess) {
        err = cuda_msg(e, "cudaHostAlloc(tables)");
        return MC_ERR_NOMEM;
    }
    std::memcpy(d.h_blob, P.buf.data(), d.blob_bytes);
    for (auto &f : P.fix) *f.first = static_cast<const char *>(d.blob) + f.second;
    mc_status us = upload_tables(d, err);
    if (us != MC_OK) return us;

    const size_t nb = (size_t)std::max<int64_t>(t.n_bins(), 1);
    if ((e = cudaMalloc(&d.d_sum, nb * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&d.d_sq, nb * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&d.d_exact, nb * 2 * kExactLimbs * sizeof(long long))) != cudaSuccess) {
        err = cuda_msg(e, "cudaMalloc(tallies)");
        return MC_ERR_NOMEM;
    }
    d.ready = true;
    return reset_tallies(d, err);
}

void device_problem_free(DeviceProblem &d)
{
    if (d.stream) cudaStreamSynchronize(d.stream);
    event_state_free(d.ev_state);
    d.ev_state = nullptr;
    bank_state_free(d.bank_state);
    d.bank_state = nullptr;
    lr_scratch_free(d.lr);
    d.lr = nullptr;
    devbuf_free(d.hist); devbuf_free(d.stack); devbuf_free(d.digest); devbuf_free(d.misc);
    if (d.blob) cudaFree(d.blob);
    if (d.h_blob) cudaFreeHost(d.h_blob);
    if (d.d_sum) cudaFree(d.d_sum);
    if (d.d_sq) cudaFree(d.d_sq);
    if (d.d_exact) cudaFree(d.d_exact);
    for (auto &ev : d.ev) if (ev) cudaEventDestroy(ev);
    if (d.stream) cudaStreamDestroy(d.stream);
    d = DeviceProblem();
}

mc_status upload_tables(DeviceProblem &d, std::string &err)
{
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d.blob, d.h_blob, d.blob_bytes, cudaMemcpyHostToDevice, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "upload tables");
        return MC_ERR_CUDA;
    }
    return MC_OK;
}

cudaError_t upload_tables_async(DeviceProblem &d, cudaStream_t st)
{
    return cudaMemcpyAsync(d.blob, d.h_blob, d.blob_bytes, cudaMemcpyHostToDevice, st);
}

cudaError_t reset_tallies_async(DeviceProblem &d, cudaStream_t st)
{
    const size_t nb = (size_t)std::max<long long>(d.dt.n_bins, 1);
    cudaError_t e;
    if ((e = cudaMemsetAsync(d.d_sum, 0, nb * sizeof(double), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d.d_sq, 0, nb * sizeof(double), st)) != cudaSuccess ||
        (e = cudaMemsetAsync(d.d_exact, 0, nb * 2 * kExactLimbs * sizeof(long long), st)) != cudaSuccess)
        return e;
    d.exact_valid = true;
    d.histories = 0;
    d.ntrack = 0;
    return cudaSuccess;
}

mc_status reset_tallies(DeviceProblem &d, std::string &err)
{
    const size_t nb = (size_t)std::max<long long>(d.dt.n_bins, 1);
    cudaError_t e;
    if ((e = cudaMemsetAsync(d.d_sum, 0, nb * sizeof(double), d.stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(d.d_sq, 0, nb * sizeof(double), d.stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(d.d_exact, 0, nb * 2 * kExactLimbs * sizeof(long long), d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "reset tallies");
        return MC_ERR_CUDA;
    }
    d.exact_valid = true;
    d.histories = 0;
    d.ntrack = 0;
    return MC_OK;
}

mc_status read_sums(const DeviceProblem &d, std::vector<double> &sum, std::vector<double> &sq, std::string &err)
{
    const size_t nb = (size_t)std::max<long long>(d.dt.n_bins, 1);
    sum.assign(nb, 0.0);
    sq.assign(nb, 0.0);
    cudaError_t e;
    if ((e = cudaStreamSynchronize(d.stream)) != cudaSuccess ||
        (e = cudaMemcpy(sum.data(), d.d_sum, nb * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(sq.data(), d.d_sq, nb * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) {
        err = cuda_msg(e, "read tallies");
        return MC_ERR_CUDA;
    }
    return MC_OK;
}

mc_status run_histories(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed,
                        mc_mode mode, const mc_tune *tune, std::string &err)
{
    std::memset(&d.last, 0, sizeof(d.last));
    if (n == 0) return MC_OK;
    if (mode == MC_MIXED_EVENT) return run_event(t, d, first, n, seed, tune, err);
    return run_fp64(t, d, first, n, seed, mode == MC_FP64_REPLAY, tune, err);
}

mc_status run_fp64(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed, bool replay,
                   const mc_tune *tune, std::string &err)
{
    const int block = (tune && tune->block) ? (int)tune->block : 128;
    if (block != 128) { err = "FP64 history kernels are built for 128-thread blocks"; return MC_ERR_ARG; }
    uint32_t depth = (tune && tune->stack_depth) ? tune->stack_depth : 32;
    // a combed bank holds `teeth` particles plus the split copies of one walk
    if (t.comb_teeth > 0 && !(tune && tune->stack_depth)) depth = std::max<uint32_t>(depth, (uint32_t)t.comb_teeth + 32);
    const bool want_digest = tune && tune->record_digests;
    int max_threads = history_fp64_max_threads(replay, block);
    int grid = (tune && tune->grid_blocks) ? (int)tune->grid_blocks : max_threads / block;
    if (grid < 1) grid = 1;
    const long long nb = std::max<long long>(d.dt.n_bins, 1);
    // chunk: histories whose per-history rows are kept before the fold;
    // bounded to ~1 GiB of rows
    uint64_t chunk = (tune && tune->chunk) ? tune->chunk : (uint64_t)((1ull << 30) / (nb * sizeof(double)));
    chunk = std::max<uint64_t>(1, std::min<uint64_t>(chunk, 1u << 22));
    chunk = std::min<uint64_t>(chunk, n);
    const uint64_t threads = (uint64_t)grid * block;
    if (!devbuf_reserve(d.hist, (size_t)chunk * nb * sizeof(double)) ||
        !devbuf_reserve(d.stack, (size_t)threads * depth * fp64_particle_bytes()) ||
        !devbuf_reserve(d.misc, 256 + kNumCounters * sizeof(unsigned long long) + 64) ||
        (want_digest && !devbuf_reserve(d.digest, (size_t)chunk * sizeof(uint64_t)))) {
        err = "cannot allocate FP64 scratch";
        return MC_ERR_NOMEM;
    }
    char *misc = static_cast<char *>(d.misc.ptr);
    unsigned long long *d_cnt = reinterpret_cast<unsigned long long *>(misc);
    int *d_status = reinterpret_cast<int *>(misc + kNumCounters * sizeof(unsigned long long));
    unsigned int *d_next = reinterpret_cast<unsigned int *>(misc + kNumCounters * sizeof(unsigned long long) + 16);
    cudaError_t e;
    if ((e = cudaMemsetAsync(misc, 0, 256 + kNumCounters * sizeof(unsigned long long), d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "memset");
        return MC_ERR_CUDA;
    }
    if (want_digest) d.digests.assign(n, 0);
    else d.digests.clear();

    float t_transport = 0.f, t_fold = 0.f;
    uint32_t launches = 0;
    // the exact sums stay valid only if this run completes
    const bool exact_was_valid = d.exact_valid;
    d.exact_valid = false;
    cudaEventRecord(d.ev[0], d.stream);
    for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
        const uint32_t cn = (uint32_t)std::min<uint64_t>(chunk, n - c0);
        HistoryArgs A;
        A.first = first + c0;
        A.n = cn;
        A.seed = seed;
        A.hist = static_cast<double *>(d.hist.ptr);
        A.stack = d.stack.ptr;
        A.stack_depth = depth;
        if (tune && tune->max_events) A.max_events = tune->max_events;
        A.counters = d_cnt;
        A.digest = want_digest ? static_cast<unsigned long long *>(d.digest.ptr) : nullptr;
        A.status = d_status;
        A.next = d_next;
        cudaMemsetAsync(d_next, 0, sizeof(unsigned int), d.stream);
        cudaEventRecord(d.ev[1], d.stream);
        if ((e = launch_history_fp64(d.dt, A, replay, grid, block, d.stream)) != cudaSuccess) {
            err = cuda_msg(e, "history kernel launch");
            return MC_ERR_CUDA;
        }
        cudaEventRecord(d.ev[2], d.stream);
        if ((e = launch_fold(A.hist, cn, d.dt.n_bins, d.d_sum, d.d_sq, replay, d.stream)) != cudaSuccess ||
            (e = launch_fold_exact(A.hist, cn, d.dt.n_bins, d.d_exact, d.stream)) != cudaSuccess) {
            err = cuda_msg(e, "fold kernel launch");
            return MC_ERR_CUDA;
        }
        cudaEventRecord(d.ev[3], d.stream);
        launches += 3;
        if (want_digest) {
            cudaMemcpyAsync(d.digests.data() + c0, A.digest, cn * sizeof(uint64_t), cudaMemcpyDeviceToHost, d.stream);
        }
        int hs = 0;
        if ((e = cudaMemcpyAsync(&hs, d_status, sizeof(int), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
            err = cuda_msg(e, "history kernel");
            return MC_ERR_CUDA;
        }
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, d.ev[1], d.ev[2]);
        cudaEventElapsedTime(&b, d.ev[2], d.ev[3]);
        t_transport += a;
        t_fold += b;
        if (hs != DS_OK) {
            err = device_status_text(hs);
            if (hs == DS_OVERFLOW) err += " (raise mc_tune.stack_depth)";
            return status_from_device(hs);
        }
    }
    if ((e = launch_exact_normalize(d.d_exact, d.dt.n_bins, d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "exact sums");
        return MC_ERR_CUDA;
    }
    ++launches;
    float total = 0.f;
    cudaEventRecord(d.ev[3], d.stream);
    cudaStreamSynchronize(d.stream);
    cudaEventElapsedTime(&total, d.ev[0], d.ev[3]);
    unsigned long long cnt[kNumCounters];
    if ((e = cudaMemcpy(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost)) != cudaSuccess) {
        err = cuda_msg(e, "counters");
        return MC_ERR_CUDA;
    }
    mc_counters &L = d.last;
    L.flights = cnt[0]; L.collisions = cnt[1]; L.crossings = cnt[2]; L.tally_updates = cnt[3];
    L.particles = cnt[4]; L.splits = cnt[5]; L.xs_evals = cnt[6]; L.freegas_iters = cnt[7];
    L.nuc_lookups = cnt[8];
    L.histories = n;
    L.transport_ms = t_transport;
    L.fold_ms = t_fold;
    L.total_ms = total;
    L.launches = launches;
    d.histories += n;
    d.ntrack += L.flights;
    d.exact_valid = exact_was_valid;
    return MC_OK;
}

}  // namespace mc
