// mc_event.cu -- mixed-precision transport engine: host side (tables on the
// device, launch shapes, scratch, single-problem runs and batches of
// problems replayed from a CUDA graph) and the tile kernel's instantiations.
// The device code is in mc_event_kernels.cuh.
//
// The reference walks one particle at a time through general.cpp:177-211.
// Two persistent kernels do the same walk here, with the same event
// functions and the same random-number keying, so they follow the same
// tracks:
//
//   k_track  one particle per thread, in registers: advance (cross-section
//            lookup, distance to collision and to the cell's surfaces,
//            flight, track-length tallies), then the collision (collision
//            tallies, implicit capture, scatter nuclide, free-gas target
//            sampled by the whole warp at once, weight roulette) or the
//            crossing (new cell, boundary condition, crossing tallies,
//            importance roulette / splitting).  Split copies wait on the
//            thread's own stack; a thread takes the next history with one
//            atomic per warp.  Built in flavours (continuous energy,
//            multigroup, everything) so that each problem runs a kernel
//            without the code it cannot use.
//   k_event  a tile of particles per CTA as a structure of arrays in shared
//            memory, advanced one event per iteration: refill + advance,
//            then the collision and crossing queues (warp ballot + popc
//            compaction), with the split copies in a per-CTA overflow bank.
//
// Tracking is FP32: positions, directions, energy, weight, distances and
// cross-section interpolation.  Sphere and cylinder roots take the constant
// term |p - c|^2 - r^2 as a compensated FP32 pair (error-free products and
// sums) where cancellation bites, and use the stable quadratic form.  The
// surface just crossed is known exactly ("coincident" surface) instead of the
// reference's FLT_EPSILON nudge and all-cell search (general.cpp:94-96),
// which FP32 positions cannot resolve: the new cell is searched among the
// cells that list that surface with the opposite sense.  Tallies accumulate
// in FP64: per history into L2-resident rows with a touched-bin mask, folded
// into per-CTA shared sums when the history's last particle dies, and into
// the global sums once per CTA.  Physics and tally semantics follow the
// reference line by line as the FP64 path does (see mc_history.cu); only the
// precision and the crossing logic differ, so results agree statistically,
// not bit for bit.
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "mc_engine.h"
#include "mc_event_kernels.cuh"

namespace mc {
using namespace ev;

struct EventState {
    EvHost host;
    void *d_blob = nullptr;
    void *h_blob = nullptr;       // pinned copy of host.blob: mc_problem_upload copies it again
    size_t blob_bytes = 0;
    EvTables dv{};
    DevBuf acc, mask, ovf, misc;
    int grid = 0, block = 0, tile = 0, ovf_cap = 0;
    size_t smem = 0;
    bool rows_dirty = true;
    // a problem whose sums do not fit in shared memory: replicas of its
    // sums ([2][n_rep][n_bins]) and what k_batch_reduce reads for one
    // problem (the sums' pointers, rep_off = {0, n_bins}, rep_prob = 0)
    DevBuf rep, rep_meta;
    int n_rep = 0;
    long long rep_stride = 0;
    bool rep_dirty = false;
};

void event_state_free(EventState *s)
{
    if (!s) return;
    if (s->d_blob) cudaFree(s->d_blob);
    if (s->h_blob) cudaFreeHost(s->h_blob);
    devbuf_free(s->acc);
    devbuf_free(s->mask);
    devbuf_free(s->ovf);
    devbuf_free(s->misc);
    devbuf_free(s->rep);
    devbuf_free(s->rep_meta);
    delete s;
}

namespace {

size_t tile_smem_bytes(int P, long long nb_smem)
{
    // the layout of Tile: hidx, the four-byte arrays, qc / qx, the sums
    return (size_t)P * (8 + 4 * TA_COUNT + 2 * sizeof(unsigned short)) + sizeof(double) * 2 * (size_t)nb_smem + 64;
}

// The replicas of a batch's sums into each problem's sums (fixed order over
// the replicas), and the replicas back to zero for the next run.
__global__ void k_batch_reduce(const EvArgs A, const int *rep_prob)
{
    const long long stride = A.rep_stride;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < stride;
         j += (long long)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0;
        for (int k = 0; k < A.n_rep; ++k) {
            const size_t at = (size_t)k * (size_t)stride + (size_t)j;
            s += A.rsum[at];
            q += A.rsq[at];
            A.rsum[at] = 0.0;
            A.rsq[at] = 0.0;
        }
        if (s != 0.0 || q != 0.0) {
            const int p = rep_prob[j];
            const long long bin = j - A.rep_off[p];
            A.psum[p][bin] += s;
            A.psq[p][bin] += q;
        }
    }
}

EvKernel pick_kernel(int minb, bool batch, int kernel, int flavor)
{
    if (kernel == 2) {
        if (flavor == FL_CE) return pick_track_ce(minb, batch);
        if (flavor == FL_MG) return pick_track_mg(minb, batch);
        return pick_track_all(minb, batch);
    }
    if (batch) {
        switch (minb) {
        case 2: return k_event<2, true>;
        case 3: return k_event<3, true>;
        default: return k_event<4, true>;
        }
    }
    switch (minb) {
    case 2: return k_event<2, false>;
    case 3: return k_event<3, false>;
    default: return k_event<4, false>;
    }
}

}  // namespace

bool event_tables_ready(const Tables &t, DeviceProblem &d, std::string &err)
{
    if (d.ev_state) return true;
    EventState *S = new EventState();
    if (!build_event_tables(t, S->host, err)) { delete S; return false; }
    cudaError_t e;
    S->blob_bytes = std::max<size_t>(S->host.blob.size(), 16);
    S->host.blob.resize(S->blob_bytes);
    if ((e = cudaMalloc(&S->d_blob, S->blob_bytes)) != cudaSuccess ||
        (e = cudaHostAlloc(&S->h_blob, S->blob_bytes, cudaHostAllocDefault)) != cudaSuccess) {
        event_state_free(S);
        err = cuda_msg(e, "allocating the event tables");
        return false;
    }
    std::memcpy(S->h_blob, S->host.blob.data(), S->blob_bytes);
    if ((e = cudaMemcpyAsync(S->d_blob, S->h_blob, S->blob_bytes, cudaMemcpyHostToDevice, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        event_state_free(S);
        err = cuda_msg(e, "uploading the event tables");
        return false;
    }
    for (auto &f : S->host.fix) *f.first = static_cast<const char *>(S->d_blob) + f.second;
    S->dv = S->host.view;
    d.ev_state = S;
    return true;
}

mc_status event_tables_upload(DeviceProblem &d, std::string &err)
{
    if (!d.ev_state) return MC_OK;   // the mixed-precision engine has not run yet
    const EventState &S = *d.ev_state;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(S.d_blob, S.h_blob, S.blob_bytes, cudaMemcpyHostToDevice, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "upload event tables");
        return MC_ERR_CUDA;
    }
    return MC_OK;
}

cudaError_t event_tables_upload_async(DeviceProblem &d, cudaStream_t st)
{
    if (!d.ev_state) return cudaSuccess;   // the mixed-precision engine has not run yet
    const EventState &S = *d.ev_state;
    return cudaMemcpyAsync(S.d_blob, S.h_blob, S.blob_bytes, cudaMemcpyHostToDevice, st);
}

size_t event_table_bytes(const DeviceProblem &d) { return d.ev_state ? d.ev_state->blob_bytes : 0; }

const EvTables &event_tables_view(const DeviceProblem &d) { return d.ev_state->dv; }

// A batch folds its histories into kBatchReplicas copies of its sums (fewer
// where the copies would take more than kBatchReplicaBytes): one copy per
// group of CTAs, added into the problems' sums after the launch.
constexpr long long kBatchReplicas = 64;
constexpr size_t kBatchReplicaBytes = (size_t)256 << 20;

// Launch geometry of the event kernel for a tune (0 fields = tuned / defaults).
struct EvLaunch {
    int block = 256, tile = 512, minb = 4, grid = 0;
    int kernel = 1;         // 1: tile / event queues (k_event), 2: one particle per thread (k_track)
    int ovf_cap = 0;        // split-copy slots per CTA
    int flavor = FL_ALL;    // per-thread kernel flavour (FL_ALL / FL_CE / FL_MG)
    uint32_t max_events = kMaxEvents;
    int refill = 1;         // k_track: idle lanes a warp gathers before it starts histories
    size_t smem = 0;
};

static mc_status event_launch_shape(const DeviceProblem &d, const mc_tune *tune, const mc_tune &tuned,
                                    long long nb_smem, bool batch, int flavor, int comb_teeth, EvLaunch &L,
                                    std::string &err)
{
    L.flavor = flavor;
    // measured: 4 idle lanes for continuous-energy histories (~115 events),
    // 8 for the short multigroup ones
    const int refill_default = flavor == FL_MG ? 8 : 4;
    L.refill = (tune && tune->refill) ? (int)tune->refill : (tuned.refill ? (int)tuned.refill : refill_default);
    if (L.refill < 1 || L.refill > 32) { err = "refill must be 1..32"; return MC_ERR_ARG; }
    L.kernel = (tune && tune->kernel) ? (int)tune->kernel : (tuned.kernel ? (int)tuned.kernel : 2);
    if (L.kernel < 1 || L.kernel > 3) {
        err = "kernel must be 1 (tile), 2 (per thread) or 3 (event kernels over an HBM bank)";
        return MC_ERR_ARG;
    }
    if (L.kernel == 3 && (batch || comb_teeth > 0)) {
        // the event-split engine runs one problem and keeps no per-history bank
        if (tune && tune->kernel) {
            err = batch ? "the event-split engine (kernel 3) runs single problems, not batches"
                        : "the particle comb needs a per-history bank: the per-thread kernel (kernel 2) or the FP64 modes";
            return MC_ERR_ARG;
        }
        L.kernel = 2;   // a tuned kernel-3 shape does not apply here
    }
    if (L.kernel == 3) {
        L.block = 256;
        L.tile = (tune && tune->bank_capacity) ? (int)tune->bank_capacity
               : ((tuned.kernel == 3 && tuned.bank_capacity) ? (int)tuned.bank_capacity : 0);
        return MC_OK;   // run_bank sizes the bank and the grids
    }
    if (comb_teeth > 0 && L.kernel != 2) {
        // the comb acts on one history's bank after each walk; the tile
        // kernel runs a history's particles side by side and has no such bank
        if (tune && tune->kernel) {
            err = "the particle comb needs a per-history bank: the per-thread kernel (kernel 2) or the FP64 modes";
            return MC_ERR_ARG;
        }
        L.kernel = 2;   // a tuned tile shape does not apply to a combed problem
    }
    const int block = L.kernel == 2 ? kTrackBlock : 256;
    L.block = (tune && tune->block) ? (int)tune->block : block;
    if (L.block != block) {
        err = L.kernel == 2 ? "the per-thread kernel is built for 128-thread blocks"
                            : "the tile kernel is built for 256-thread blocks";
        return MC_ERR_ARG;
    }
    const bool own_minb = tune && tune->blocks_per_sm;
    L.minb = own_minb ? (int)tune->blocks_per_sm
           : ((tuned.blocks_per_sm && tuned.kernel == (uint32_t)L.kernel) ? (int)tuned.blocks_per_sm
                                                                          : (L.kernel == 2 ? 8 : 4));
    if (L.kernel == 2 ? !(L.minb == 4 || L.minb == 6 || L.minb == 7 || L.minb == 8) : (L.minb < 2 || L.minb > 4)) {
        err = L.kernel == 2 ? "blocks_per_sm must be 4, 6, 7 or 8 for the per-thread kernel"
                            : "blocks_per_sm must be 2, 3 or 4 for the tile kernel";
        return MC_ERR_ARG;
    }
    if (L.kernel == 2) {
        L.tile = kTrackBlock;                  // one history row per thread
        // a combed stack holds `teeth` particles plus the split copies of one walk
        const int depth = (tune && tune->stack_depth) ? (int)tune->stack_depth
                                                      : std::max(kTrackDepth, comb_teeth + kTrackDepth);
        if (depth < 1 || depth > 4096) {
            err = comb_teeth > 0 && !(tune && tune->stack_depth)
                      ? "the per-thread kernel keeps at most 4064 comb teeth"
                      : "stack_depth must be 1..4096";
            return MC_ERR_ARG;
        }
        L.ovf_cap = kTrackBlock * depth;
        // the per-CTA sums, then (multigroup, with them) every thread's
        // running sums of its register bin and that bin
        L.smem = sizeof(double) * 2 * (size_t)nb_smem + 64;
        if (nb_smem > 0 && flavor == FL_MG) L.smem += kTrackBlock * (2 * sizeof(double) + sizeof(int));
    } else {
        L.tile = (tune && tune->bank_capacity) ? (int)tune->bank_capacity
               : (tuned.bank_capacity ? (int)tuned.bank_capacity : 512);
        if (L.tile < L.block || L.tile % L.block != 0 || L.tile > 4096) {
            err = "tile (bank_capacity) must be a multiple of 256 up to 4096";
            return MC_ERR_ARG;
        }
        // split copies waiting in the CTA's overflow bank: stack_depth slots
        // when given (a small bank exercises the overflow status), else 4 per
        // tile particle
        L.ovf_cap = (tune && tune->stack_depth) ? (int)tune->stack_depth : 4 * L.tile;
        if (L.ovf_cap < 1 || L.ovf_cap > (1 << 20)) {
            err = "stack_depth (the tile kernel's overflow bank) must be 1..2^20";
            return MC_ERR_ARG;
        }
        L.smem = tile_smem_bytes(L.tile, nb_smem);
    }
    EvKernel k = pick_kernel(L.minb, batch, L.kernel, L.flavor);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem)) != cudaSuccess) {
        err = cuda_msg(e, "event kernel shared memory");
        return MC_ERR_ARG;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, L.block, L.smem);
    if (per_sm < 1) { err = "event kernel does not fit on an SM with this tile"; return MC_ERR_ARG; }
    per_sm = std::min(per_sm, L.minb);
    L.grid = (tune && tune->grid_blocks) ? (int)tune->grid_blocks : d.sms * per_sm;
    return MC_OK;
}

static mc_status event_scratch(EventState &S, cudaStream_t st, int grid, int tile, int ovf_cap, long long row_nb,
                               std::string &err)
{
    const int nw = (int)((row_nb + 63) / 64);
    const size_t rows = (size_t)grid * tile;
    const size_t acc_bytes = rows * row_nb * sizeof(double);
    const size_t mask_bytes = rows * nw * sizeof(unsigned long long);
    const bool grow = !S.acc.ptr || S.acc.bytes < acc_bytes || S.mask.bytes < mask_bytes;
    if (!devbuf_reserve(S.acc, acc_bytes) || !devbuf_reserve(S.mask, mask_bytes) ||
        !devbuf_reserve(S.ovf, (size_t)grid * ovf_cap * sizeof(OvfP)) ||
        !devbuf_reserve(S.misc, 256 + kNumCounters * sizeof(unsigned long long))) {
        err = "cannot allocate event-engine scratch";
        return MC_ERR_NOMEM;
    }
    if (grow || S.rows_dirty) {
        cudaMemsetAsync(S.acc.ptr, 0, S.acc.bytes, st);
        cudaMemsetAsync(S.mask.ptr, 0, S.mask.bytes, st);
        S.rows_dirty = false;
    }
    return MC_OK;
}

static const char *status_text(int hs)
{
    return hs == DS_LOST ? "a particle was lost (no cell contains it)"
         : hs == DS_OVERFLOW ? "split-particle bank or time-filter buffer overflow"
         : hs == DS_TIMEOUT ? "a particle exceeded the event limit or the free-gas loop did not converge"
         : hs == DS_NAN ? "a non-finite track length, energy or weight" : "device error status";
}

static void fill_counters(mc_counters &L, const unsigned long long *cnt)
{
    L.flights = cnt[0]; L.collisions = cnt[1]; L.crossings = cnt[2]; L.tally_updates = cnt[3];
    L.particles = cnt[4]; L.splits = cnt[5]; L.xs_evals = cnt[6]; L.freegas_iters = cnt[7];
    L.nuc_lookups = cnt[8];
}

// Replicas of a single problem's sums when they do not fit in shared
// memory (see EvArgs::n_rep); fills A's replica fields.
static mc_status single_replicas(EventState &S, const DeviceProblem &d, long long nb, EvArgs &A,
                                 const int *&rep_prob, std::string &err)
{
    const int n_rep = (int)std::max<long long>(
        1, std::min<long long>(kBatchReplicas, (long long)(kBatchReplicaBytes / (2 * sizeof(double) * (size_t)nb))));
    const size_t rep_bytes = 2 * sizeof(double) * (size_t)n_rep * (size_t)nb;
    const size_t meta_bytes = 256 + (size_t)nb * sizeof(int);
    if (!S.rep.ptr || S.n_rep != n_rep || S.rep_stride != nb) {
        if (!devbuf_reserve(S.rep, rep_bytes) || !devbuf_reserve(S.rep_meta, meta_bytes)) {
            err = "cannot allocate the replicated sums";
            return MC_ERR_NOMEM;
        }
        S.n_rep = n_rep;
        S.rep_stride = nb;
        S.rep_dirty = true;
    }
    // the sums' pointers and rep_off = {0, nb} in the first 256 bytes, then rep_prob = 0
    struct { double *ps, *pq; long long off[2]; } h{d.d_sum, d.d_sq, {0, nb}};
    char *m = static_cast<char *>(S.rep_meta.ptr);
    cudaMemcpyAsync(m, &h, sizeof(h), cudaMemcpyHostToDevice, d.stream);
    if (S.rep_dirty) {
        cudaMemsetAsync(m + 256, 0, (size_t)nb * sizeof(int), d.stream);
        cudaMemsetAsync(S.rep.ptr, 0, rep_bytes, d.stream);
        S.rep_dirty = false;
    }
    A.rsum = static_cast<double *>(S.rep.ptr);
    A.rsq = A.rsum + (size_t)n_rep * (size_t)nb;
    A.psum = reinterpret_cast<double *const *>(m);
    A.psq = reinterpret_cast<double *const *>(m + sizeof(double *));
    A.rep_off = reinterpret_cast<const long long *>(m + 2 * sizeof(double *));
    A.rep_stride = nb;
    A.n_rep = n_rep;
    rep_prob = reinterpret_cast<const int *>(m + 256);
    return MC_OK;
}

mc_status run_event(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed,
                    const mc_tune *tune, std::string &err)
{
    if (!event_tables_ready(t, d, err)) return MC_ERR_INPUT;
    EventState &S = *d.ev_state;
    const EvTables &V = S.dv;
    const long long nb = std::max<long long>(V.n_bins, 1);
    const bool smem_sums = nb <= 4096;
    EvLaunch L;
    const int comb = t.comb_teeth > 0 ? t.comb_teeth : 0;
    const int flavor = (V.has_time || comb) ? FL_ALL : (V.G > 0 ? FL_MG : FL_CE);
    mc_status st = event_launch_shape(d, tune, d.tuned, smem_sums ? nb : 0, false, flavor, comb, L, err);
    if (st != MC_OK) return st;
    if (L.kernel == 3) {
        mc_tune bt = tune ? *tune : mc_tune{};
        bt.bank_capacity = (uint32_t)L.tile;
        if (!tune) bt.max_events = 0;
        // importance splitting needs two cells of different nonzero importance
        bool may_split = false;
        double imp0 = 0.0;
        for (double imp : t.cell_imp) {
            if (imp <= 0.0) continue;
            if (imp0 == 0.0) imp0 = imp;
            else if (imp != imp0) may_split = true;
        }
        return run_bank(d, V, flavor, may_split, first, n, seed, &bt, err);
    }
    if ((st = event_scratch(S, d.stream, L.grid, L.tile, L.ovf_cap, nb, err)) != MC_OK) return st;
    char *misc = static_cast<char *>(S.misc.ptr);
    cudaMemsetAsync(misc, 0, 256 + kNumCounters * sizeof(unsigned long long), d.stream);
    EvArgs A{};
    A.first = first;
    A.n = n;
    A.seed = seed;
    A.max_events = (tune && tune->max_events) ? tune->max_events : kMaxEvents;
    A.next = reinterpret_cast<unsigned long long *>(misc);
    A.status = reinterpret_cast<int *>(misc + 8);
    A.counters = reinterpret_cast<unsigned long long *>(misc + 64);
    A.acc = static_cast<double *>(S.acc.ptr);
    A.mask = static_cast<unsigned long long *>(S.mask.ptr);
    A.nw = (int)((nb + 63) / 64);
    A.row_nb = (int)nb;
    A.ovf = static_cast<OvfP *>(S.ovf.ptr);
    A.ovf_cap = L.ovf_cap;
    A.sum = d.d_sum;
    A.sq = d.d_sq;
    A.tile = L.tile;
    A.smem_sums = smem_sums ? 1 : 0;
    A.refill_min = L.refill;
    A.n_prob = 0;
    const int *d_rep_prob = nullptr;
    if (!smem_sums && (st = single_replicas(S, d, nb, A, d_rep_prob, err)) != MC_OK) return st;
    cudaEventRecord(d.ev[0], d.stream);
    pick_kernel(L.minb, false, L.kernel, L.flavor)<<<L.grid, L.block, L.smem, d.stream>>>(V, A);
    cudaError_t e;
    if ((e = cudaGetLastError()) != cudaSuccess) {
        S.rep_dirty = A.n_rep > 0;
        err = cuda_msg(e, "event kernel launch");
        return MC_ERR_CUDA;
    }
    if (A.n_rep > 0)
        k_batch_reduce<<<(int)std::min<long long>((nb + 255) / 256, 4LL * d.sms), 256, 0, d.stream>>>(A, d_rep_prob);
    cudaEventRecord(d.ev[1], d.stream);
    int hs = 0;
    unsigned long long cnt[kNumCounters];
    if ((e = cudaMemcpyAsync(&hs, A.status, sizeof(int), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cnt, A.counters, sizeof(cnt), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "event kernel");
        S.rows_dirty = true;
        S.rep_dirty = A.n_rep > 0;
        return MC_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, d.ev[0], d.ev[1]);
    if (hs != DS_OK) {
        S.rows_dirty = true;
        err = status_text(hs);
        return status_from_device(hs);
    }
    mc_counters &C = d.last;
    fill_counters(C, cnt);
    C.histories = n;
    C.transport_ms = ms;
    C.total_ms = ms;
    C.launches = A.n_rep > 0 ? 2 : 1;
    d.histories += n;
    d.ntrack += C.flights;
    d.exact_valid = false;   // the mixed mode keeps no per-history rows to sum exactly
    return MC_OK;
}

// ---------------------------------------------------------------------------
// batches of problems in one persistent launch, replayed from a CUDA graph
// ---------------------------------------------------------------------------
struct BatchState {
    std::vector<DeviceProblem *> probs;
    std::vector<uint64_t> hist;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    DevBuf meta;                      // tabs, prefix, seeds, psum, psq, rep_off, rep_prob
    DevBuf rep;                       // the replicas of the batch's sums: [2][n_rep][rep_stride]
    int n_rep = 1;
    long long rep_stride = 1;         // bins of all problems
    bool rep_dirty = false;           // a run stopped before k_batch_reduce cleared the replicas
    EventState scratch;               // rows / mask / overflow / control
    long long row_nb = 1;
    uint64_t total = 0;
    unsigned long long *h_seeds = nullptr;   // pinned: per-problem seeds of the next run
    cudaGraphExec_t exec = nullptr;
    EvLaunch shape;
    bool have_shape = false;
    bool count_histories = true;      // false for autotuning batches
    int flavor = FL_ALL;              // per-thread kernel flavour for the whole batch
    int comb_teeth = 0;               // most comb teeth of any problem (stack depth)
    mc_counters last{};
};

void batch_state_free(BatchState *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    devbuf_free(b->meta);
    devbuf_free(b->rep);
    devbuf_free(b->scratch.acc);
    devbuf_free(b->scratch.mask);
    devbuf_free(b->scratch.ovf);
    devbuf_free(b->scratch.misc);
    if (b->h_seeds) cudaFreeHost(b->h_seeds);
    for (auto &e : b->ev) if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

uint64_t batch_problem_seed(uint64_t seed, uint32_t i) { return seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1); }

mc_status batch_create(const std::vector<const Tables *> &tabs, const std::vector<DeviceProblem *> &probs,
                       const uint64_t *hist, const std::vector<double *> *sums_to, BatchState **out,
                       std::string &err)
{
    BatchState *b = new BatchState();
    b->probs = probs;
    const uint32_t n = (uint32_t)probs.size();
    std::vector<EvTables> views(n);
    std::vector<unsigned long long> prefix(n + 1, 0);
    std::vector<double *> psum(n), psq(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (!event_tables_ready(*tabs[i], *probs[i], err)) { batch_state_free(b); err = "problem " + std::to_string(i) + ": " + err; return MC_ERR_INPUT; }
        views[i] = probs[i]->ev_state->dv;
        prefix[i + 1] = prefix[i] + hist[i];
        b->hist.push_back(hist[i]);
        psum[i] = sums_to ? (*sums_to)[2 * i] : probs[i]->d_sum;
        psq[i] = sums_to ? (*sums_to)[2 * i + 1] : probs[i]->d_sq;
        b->row_nb = std::max<long long>(b->row_nb, views[i].n_bins);
    }
    // one flavour for the launch: every problem multigroup (or every one
    // continuous energy) and none with a time filter, else the full kernel
    // (the particle comb, too, takes the full kernel)
    bool all_mg = true, all_ce = true, any_time = false;
    for (uint32_t i = 0; i < n; ++i) {
        all_mg = all_mg && views[i].G > 0;
        all_ce = all_ce && views[i].G == 0;
        any_time = any_time || views[i].has_time || views[i].comb_teeth > 0;
        b->comb_teeth = std::max(b->comb_teeth, views[i].comb_teeth);
    }
    b->flavor = any_time ? FL_ALL : (all_mg ? FL_MG : (all_ce ? FL_CE : FL_ALL));
    b->total = prefix[n];
    // replicas of every problem's bins: kBatchReplicas copies, fewer where
    // they would pass kBatchReplicaBytes
    std::vector<long long> rep_off(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i) rep_off[i + 1] = rep_off[i] + std::max<long long>(views[i].n_bins, 0);
    b->rep_stride = std::max<long long>(rep_off[n], 1);
    std::vector<int> rep_prob((size_t)b->rep_stride, 0);
    for (uint32_t i = 0; i < n; ++i)
        for (long long j = rep_off[i]; j < rep_off[i + 1]; ++j) rep_prob[(size_t)j] = (int)i;
    b->n_rep = (int)std::max<long long>(
        1, std::min<long long>(kBatchReplicas, (long long)(kBatchReplicaBytes / (2 * sizeof(double) * (size_t)b->rep_stride))));
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        batch_state_free(b);
        err = cuda_msg(e, "batch stream");
        return MC_ERR_CUDA;
    }
    for (auto &ev : b->ev) cudaEventCreate(&ev);
    const size_t sz = n * sizeof(EvTables) + (n + 1) * 8 + n * 8 + 2 * n * sizeof(double *) + (n + 1) * 8 +
                      (size_t)b->rep_stride * sizeof(int) + 8 * 256;
    const size_t rep_bytes = 2 * sizeof(double) * (size_t)b->n_rep * (size_t)b->rep_stride;
    if (!devbuf_reserve(b->meta, sz) || !devbuf_reserve(b->rep, rep_bytes) ||
        cudaHostAlloc(&b->h_seeds, n * 8, cudaHostAllocDefault) != cudaSuccess) {
        batch_state_free(b);
        err = "cannot allocate batch descriptors";
        return MC_ERR_NOMEM;
    }
    char *m = static_cast<char *>(b->meta.ptr);
    size_t off = 0;
    cudaError_t put_err = cudaSuccess;
    auto put = [&](const void *src, size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        const cudaError_t e = cudaMemcpy(m + off, src, bytes, cudaMemcpyHostToDevice);
        if (put_err == cudaSuccess) put_err = e;
        const size_t at = off;
        off += bytes;
        return at;
    };
    put(views.data(), n * sizeof(EvTables));
    put(prefix.data(), (n + 1) * 8);
    put(psum.data(), n * sizeof(double *));
    put(psq.data(), n * sizeof(double *));
    off = (off + 255) & ~(size_t)255;
    off += n * 8;   // the seeds (written by each run)
    put(rep_off.data(), (n + 1) * sizeof(long long));
    put(rep_prob.data(), (size_t)b->rep_stride * sizeof(int));
    if (put_err == cudaSuccess) put_err = cudaMemset(b->rep.ptr, 0, rep_bytes);
    if (put_err != cudaSuccess) {
        batch_state_free(b);
        err = cuda_msg(put_err, "batch descriptors");
        return MC_ERR_CUDA;
    }
    b->count_histories = sums_to == nullptr;
    *out = b;
    return MC_OK;
}

mc_status batch_run(BatchState *b, int device_sms, uint64_t seed, const mc_tune *tune, const mc_tune &tuned,
                    std::string &err)
{
    const uint32_t n = (uint32_t)b->probs.size();
    DeviceProblem shape_dev;
    shape_dev.sms = device_sms;
    EvLaunch L;
    mc_status st = event_launch_shape(shape_dev, tune, tuned, 0, true, b->flavor, b->comb_teeth, L, err);
    if (st != MC_OK) return st;
    if ((st = event_scratch(b->scratch, b->stream, L.grid, L.tile, L.ovf_cap, b->row_nb, err)) != MC_OK) return st;
    L.max_events = (tune && tune->max_events) ? tune->max_events : kMaxEvents;
    const bool same_shape = b->have_shape && L.grid == b->shape.grid && L.tile == b->shape.tile &&
                            L.minb == b->shape.minb && L.kernel == b->shape.kernel &&
                            L.max_events == b->shape.max_events && L.refill == b->shape.refill;
    for (uint32_t i = 0; i < n; ++i) b->h_seeds[i] = batch_problem_seed(seed, i);
    char *m = static_cast<char *>(b->meta.ptr);
    size_t off = 0;
    auto at = [&](size_t bytes) { off = (off + 255) & ~(size_t)255; const size_t a = off; off += bytes; return m + a; };
    const EvTables *d_tabs = reinterpret_cast<const EvTables *>(at(n * sizeof(EvTables)));
    const unsigned long long *d_prefix = reinterpret_cast<const unsigned long long *>(at((n + 1) * 8));
    double *const *d_psum = reinterpret_cast<double *const *>(at(n * sizeof(double *)));
    double *const *d_psq = reinterpret_cast<double *const *>(at(n * sizeof(double *)));
    unsigned long long *d_seeds = reinterpret_cast<unsigned long long *>(at(n * 8));
    const long long *d_rep_off = reinterpret_cast<const long long *>(at((n + 1) * sizeof(long long)));
    const int *d_rep_prob = reinterpret_cast<const int *>(at((size_t)b->rep_stride * sizeof(int)));
    double *d_rsum = static_cast<double *>(b->rep.ptr);
    double *d_rsq = d_rsum + (size_t)b->n_rep * (size_t)b->rep_stride;
    cudaError_t e;
    if (b->rep_dirty) {
        cudaMemsetAsync(b->rep.ptr, 0, 2 * sizeof(double) * (size_t)b->n_rep * (size_t)b->rep_stride, b->stream);
        b->rep_dirty = false;
    }
    if (!same_shape) {
        if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        char *misc = static_cast<char *>(b->scratch.misc.ptr);
        EvArgs A{};
        A.first = 0;
        A.n = b->total;
        A.seed = 0;
        A.max_events = L.max_events;
        A.next = reinterpret_cast<unsigned long long *>(misc);
        A.status = reinterpret_cast<int *>(misc + 8);
        A.counters = reinterpret_cast<unsigned long long *>(misc + 64);
        A.acc = static_cast<double *>(b->scratch.acc.ptr);
        A.mask = static_cast<unsigned long long *>(b->scratch.mask.ptr);
        A.nw = (int)((b->row_nb + 63) / 64);
        A.row_nb = (int)b->row_nb;
        A.ovf = static_cast<OvfP *>(b->scratch.ovf.ptr);
        A.ovf_cap = L.ovf_cap;
        A.tile = L.tile;
        A.smem_sums = 0;
        A.refill_min = L.refill;
        A.tabs = d_tabs;
        A.prefix = d_prefix;
        A.seeds = d_seeds;
        A.psum = d_psum;
        A.psq = d_psq;
        A.n_prob = (int)n;
        A.rsum = d_rsum;
        A.rsq = d_rsq;
        A.rep_off = d_rep_off;
        A.rep_stride = b->rep_stride;
        A.n_rep = b->n_rep;
        EvTables V0{};
        V0.n_bins = 0;
        // capture: seeds (pinned host -> device), control reset, the launch
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
            err = cuda_msg(e, "graph capture");
            return MC_ERR_CUDA;
        }
        cudaMemcpyAsync(d_seeds, b->h_seeds, n * 8, cudaMemcpyHostToDevice, b->stream);
        cudaMemsetAsync(misc, 0, 256 + kNumCounters * sizeof(unsigned long long), b->stream);
        pick_kernel(L.minb, true, L.kernel, L.flavor)<<<L.grid, L.block, L.smem, b->stream>>>(V0, A);
        const int rgrid = (int)std::min<long long>((b->rep_stride + 255) / 256, 4LL * device_sms);
        k_batch_reduce<<<rgrid, 256, 0, b->stream>>>(A, d_rep_prob);
        if ((e = cudaStreamEndCapture(b->stream, &g)) != cudaSuccess) {
            err = cuda_msg(e, "graph capture end");
            return MC_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { err = cuda_msg(e, "graph instantiate"); return MC_ERR_CUDA; }
        b->shape = L;
        b->have_shape = true;
    }
    cudaEventRecord(b->ev[0], b->stream);
    if ((e = cudaGraphLaunch(b->exec, b->stream)) != cudaSuccess) {
        b->rep_dirty = true;
        err = cuda_msg(e, "graph launch");
        return MC_ERR_CUDA;
    }
    cudaEventRecord(b->ev[1], b->stream);
    char *misc = static_cast<char *>(b->scratch.misc.ptr);
    int hs = 0;
    unsigned long long cnt[kNumCounters];
    if ((e = cudaMemcpyAsync(&hs, misc + 8, sizeof(int), cudaMemcpyDeviceToHost, b->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cnt, misc + 64, sizeof(cnt), cudaMemcpyDeviceToHost, b->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(b->stream)) != cudaSuccess) {
        err = cuda_msg(e, "batch kernel");
        b->scratch.rows_dirty = true;
        b->rep_dirty = true;
        return MC_ERR_CUDA;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
    if (hs != DS_OK) {
        b->scratch.rows_dirty = true;
        b->have_shape = false;    // re-capture: the row memset must run first
        err = status_text(hs);
        return status_from_device(hs);
    }
    std::memset(&b->last, 0, sizeof(b->last));
    fill_counters(b->last, cnt);
    b->last.histories = b->total;
    b->last.transport_ms = ms;
    b->last.total_ms = ms;
    b->last.launches = 2;   // the transport kernel and k_batch_reduce
    if (b->count_histories)
        for (uint32_t i = 0; i < n; ++i) {
            b->probs[i]->histories += b->hist[i];
            b->probs[i]->exact_valid = false;
        }
    return MC_OK;
}

cudaStream_t batch_stream(const BatchState *b) { return b->stream; }

const mc_counters &batch_counters(const BatchState *b) { return b->last; }

}  // namespace mc
