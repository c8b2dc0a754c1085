// mc_bank.cu -- the mixed-precision mode's event-split engine (mc_tune.kernel
// = 3): the particle bank as a structure of arrays in HBM and one kernel per
// event type over queues compacted with warp ballots and prefix sums.
//
// The reference walks one particle through general.cpp:177-211 until it
// dies.  Here every live particle of the bank takes one event per iteration,
// and each iteration is three launches over the bank:
//
//   k_bank_advance  every slot of the bank, in slot order.  An empty slot is
//                   refilled first (a waiting split copy, else a new history
//                   whose tally row is this slot's own row), then every
//                   particle takes its flight: cross-section lookup,
//                   distance to collision and to the cell's surfaces,
//                   track-length tallies (general.cpp:40-83).  Each particle
//                   is appended to the collision queue or the crossing
//                   queue.
//   k_bank_collide  the collision queue: collision tallies, implicit capture,
//                   scatter nuclide, the free-gas target sampled by the whole
//                   warp at once, weight roulette (general.cpp:121-163,
//                   population_control.cpp:9-15).
//   k_bank_cross    the crossing queue: boundary condition, new cell,
//                   crossing tallies, importance roulette / splitting
//                   (general.cpp:89-115, population_control.cpp:21-49); split
//                   copies wait in an HBM stack.  The last block to finish
//                   closes the iteration (empties the queues, decides
//                   whether the run is done).
//
// A particle stays in its slot from birth to death; a flag per slot says
// whether it holds one, and a dead particle's slot is refilled by the next
// advance.  Every queue append is one atomic per warp: a ballot gives the
// lanes that append and their prefix count gives each lane its place.  A
// particle's state is read and written as 16-byte vectors (position +
// weight, direction + energy, cell / surface / group / row) at its slot, so
// the advance kernel's accesses, in slot order, coalesce.  The event
// functions and the random-number keying are the other mixed-precision
// kernels' (mc_event_kernels.cuh), so a particle follows the same track here
// as in k_track and k_event.
//
// Tallies: a history's tallies go to the tally row of the slot that started
// it, as reductions in L2; when its last particle dies the row's touched bins
// are folded into the global sums (Estimator.cpp:339-346).  A slot whose row
// still belongs to a live history (split copies of it elsewhere) takes only
// split copies until that history ends.
//
// Problems with the particle comb are refused (the comb acts on one
// history's bank after each walk; this engine keeps none), as are batches.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "mc_engine.h"
#include "mc_event_kernels.cuh"

namespace mc {
using namespace ev;

namespace {

constexpr int kBankBlock = 256;
constexpr int kBankDefault = 1 << 20;    // particle slots (and tally rows)
constexpr int kIterPerCheck = 32;        // iterations between two host checks

struct BankCtl {
    unsigned long long next;     // histories handed out (relative to first)
    int n_live;                  // slots holding a particle
    int n_coll, n_cross;         // this iteration's queues
    int n_split;                 // split copies waiting
    int status;
    unsigned int blocks_done;    // k_bank_cross blocks finished
    int done;
    unsigned int iter;
    int pad[2];
};

struct BankArgs {
    float4 *pw;          // x, y, z, weight
    float4 *dE;          // u, v, w, E
    int4 *meta;          // cell, last crossed surface, group, tally row
    uint2 *idev;         // particle id, events taken
    float *t;            // time (problems with a time filter)
    float4 *fx;          // advance -> collide: Sigma_t, Sigma_s, Sigma_c, grid fraction
    int2 *fl;            // advance -> collide / cross: grid index, surface << 2 | (sense + 1)
    int *live;           // [P] the slot holds a particle
    int *qc, *qx;        // collision / crossing queues (slot indices)
    OvfP *split;         // split copies waiting (a stack)
    int split_cap;
    int P;               // slots
    unsigned long long *hidx;   // [P] history of the row
    int *hlive;                 // [P] the row's history: particles alive or waiting
    BankCtl *ctl;
    unsigned long long *bcnt;   // [grid][kNumCounters] per-block event counters
    int may_split;              // cells differ in importance: a history may own several particles
};

// sums: the block's shared tally sums (2 x n_bins doubles; nullptr = the
// global sums take each history's fold directly)
__device__ __forceinline__ void bank_ctx(Ctx &C, const EvTables &V, const EvArgs &A, uint32_t *s_cnt, int *s_status,
                                         double *sums = nullptr)
{
    C.V = &V;
    C.A = &A;
    C.T.base = reinterpret_cast<unsigned char *>(sums);
    C.T.P = 0;
    C.T.nsum = sums ? V.n_bins : 0;
    C.s_status = s_status;
    C.s_novf = nullptr;
    C.s_nlive = nullptr;
    C.s_nhfree = nullptr;
    C.reg_mask = false;
    C.tmask = 0ull;
    C.tmask1 = 0ull;
    C.cbin = -1;
    C.cval = 0.0;
    C.cnt.base = cnt_column(s_cnt, threadIdx.x);
    for (int i = 0; i < kNumCounters; ++i) C.cnt[i] = 0;
}

// The block's event counters into its own slot of the per-block array (one
// block of a launch per slot: plain adds, no contention), and its status.
__device__ __forceinline__ void bank_flush(const BankArgs &B, uint32_t *s_cnt, int s_status,
                                           const EvArgs *A = nullptr, const double *sums = nullptr, long long nb = 0)
{
    __syncthreads();
    if (sums) {   // the block's folded histories, one global atomic per nonzero bin
        for (long long b = threadIdx.x; b < nb; b += blockDim.x) {
            const double sv = sums[b], qv = sums[nb + b];
            if (sv != 0.0) atomicAdd(A->sum + b, sv);
            if (qv != 0.0) atomicAdd(A->sq + b, qv);
        }
    }
    __shared__ unsigned long long s_red[kBankBlock / 32][kNumCounters];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = 0; i < kNumCounters; ++i) {
        unsigned long long v = cnt_column(s_cnt, threadIdx.x)[i * kCntStride];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) s_red[warp][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < kNumCounters) {
        unsigned long long v = 0;
        for (int w = 0; w < kBankBlock / 32; ++w) v += s_red[w][threadIdx.x];
        if (v) B.bcnt[(size_t)blockIdx.x * kNumCounters + threadIdx.x] += v;
    }
    if (threadIdx.x == 0 && s_status != 0) atomicCAS(&B.ctl->status, 0, s_status);
}

__device__ __forceinline__ void bank_load(const BankArgs &B, const EvTables &V, int s, PState &p)
{
    const float4 a = B.pw[s], b = B.dE[s];
    const int4 m = B.meta[s];
    const uint2 ie = B.idev[s];
    p.x = a.x; p.y = a.y; p.z = a.z; p.wt = a.w;
    p.u = b.x; p.v = b.y; p.w = b.z; p.E = b.w;
    p.cell = m.x; p.surf = m.y; p.g = m.z; p.hslot = m.w;
    p.id = ie.x; p.ev = ie.y;
    p.t = V.has_time ? B.t[s] : 0.f;
    p.prob = 0;
}

__device__ __forceinline__ void bank_store(const BankArgs &B, const EvTables &V, int s, const PState &p)
{
    B.pw[s] = make_float4(p.x, p.y, p.z, p.wt);
    B.dE[s] = make_float4(p.u, p.v, p.w, p.E);
    B.meta[s] = make_int4(p.cell, p.surf, p.g, p.hslot);
    B.idev[s] = make_uint2(p.id, p.ev);
    if (V.has_time) B.t[s] = p.t;
}

// a dead particle: its slot empties (all lanes call this, for the count of
// live slots), its history's row is folded when it was the history's last
// particle
template <int kFl>
__device__ __forceinline__ void bank_retire(Ctx &C, const BankArgs &B, bool dies, int s, int hslot)
{
    const unsigned dm = __ballot_sync(0xffffffffu, dies);
    if (dm && (threadIdx.x & 31) == __ffs(dm) - 1) atomicSub(&B.ctl->n_live, __popc(dm));
    if (dies) {
        B.live[s] = 0;
        // with splitting, the history's other particles may run on other
        // SMs in this same kernel: their tally reductions must be visible
        // before the last one folds the row.  Without it the history's one
        // particle made every reduction itself, in this or an earlier kernel.
        if (B.may_split) __threadfence();
        if (atomicSub(&B.hlive[hslot], 1) == 1) {
            if (B.may_split) __threadfence();
            history_fold<kFl, false>(C, hslot, 0);
        }
    }
}

template <int kFl>
__global__ void __launch_bounds__(kBankBlock) k_bank_advance(const EvTables V, const EvArgs A, const BankArgs B)
{
    __shared__ uint32_t s_cnt[cnt_words(kBankBlock)];
    __shared__ int s_status, s_go, s_more;
    const volatile BankCtl *vc = B.ctl;
    if (threadIdx.x == 0) {
        s_status = 0;
        s_go = !(vc->done || vc->status);   // one decision for the whole block
        s_more = vc->next < A.n;            // histories left to start (it only grows)
    }
    __syncthreads();
    if (!s_go) return;
    Ctx C;
    bank_ctx(C, V, A, s_cnt, &s_status);
    const int lane = threadIdx.x & 31;
    for (int s0 = blockIdx.x * blockDim.x; s0 < B.P; s0 += gridDim.x * blockDim.x) {
        const int s = s0 + threadIdx.x;     // P is a multiple of the block
        bool live = B.live[s] != 0, fresh = false;
        PState p;
        if (live) {
            bank_load(B, V, s, p);
        } else if (*(volatile int *)&B.ctl->n_split > 0) {
            // a waiting split copy first (a stack: pops only in this kernel)
            const int k = atomicSub(&B.ctl->n_split, 1);
            if (k > 0) {
                const OvfP o = B.split[k - 1];
                p.x = o.x; p.y = o.y; p.z = o.z; p.u = o.u; p.v = o.v; p.w = o.w;
                p.E = o.E; p.wt = o.wt; p.t = o.t; p.cell = o.cell; p.surf = o.surf;
                p.hslot = o.hslot; p.g = o.g; p.id = o.id; p.ev = 0u; p.prob = 0;
                fresh = true;
                C.cnt[C_PART]++;
            } else {
                atomicAdd(&B.ctl->n_split, 1);
            }
        }
        // else a new history, in this slot's own row when that row is free
        const bool want = s_more && !live && !fresh && B.hlive[s] == 0;
        const unsigned wm = __ballot_sync(0xffffffffu, want);
        if (wm) {
            const int leader = __ffs(wm) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&B.ctl->next, (unsigned long long)__popc(wm));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                const unsigned long long gi = base + (unsigned long long)__popc(wm & ((1u << lane) - 1u));
                if (gi < A.n) {
                    const uint64_t hist = A.first + gi;
                    B.hidx[s] = hist;
                    B.hlive[s] = 1;
                    sample_source(V, A.seed, hist, p);
                    p.hslot = s;
                    fresh = true;
                    C.cnt[C_PART]++;
                }
            }
        }
        // slots filled now join the live count (one atomic per warp)
        const unsigned fm = __ballot_sync(0xffffffffu, fresh);
        if (fm) {
            if (lane == __ffs(fm) - 1) atomicAdd(&B.ctl->n_live, __popc(fm));
            if (fresh) B.live[s] = 1;
        }
        live = live || fresh;
        int kind = 0;
        if (live) {
            p.ev += 1u;
            if (p.ev > A.max_events) {        // bounded walk: report, never spin
                atomicCAS(&s_status, 0, DS_TIMEOUT);
                p.ev = A.max_events;
            }
            Rng32 R;
            R.init(A.seed, B.hidx[p.hslot], p.id, p.ev, 0u);
            Flight f;
            kind = event_advance<kFl>(C, V, R, p, f);
            // the flight moves the particle and clears its last surface; the
            // direction and energy change only for a particle placed here now
            B.pw[s] = make_float4(p.x, p.y, p.z, p.wt);
            if (fresh) B.dE[s] = make_float4(p.u, p.v, p.w, p.E);
            B.meta[s] = make_int4(p.cell, p.surf, p.g, p.hslot);
            B.idev[s] = make_uint2(p.id, p.ev);
            if (V.has_time) B.t[s] = p.t;
            if (kind != 0) {
                B.fx[s] = make_float4(f.sig, f.ss, f.sc, f.xa.f);
                B.fl[s] = make_int2(f.xa.i, (f.S << 2) | (f.sense + 1));
            }
        }
        const int pc = warp_append(&B.ctl->n_coll, kind == 1);
        if (kind == 1) B.qc[pc] = s;
        const int px = warp_append(&B.ctl->n_cross, kind == 2);
        if (kind == 2) B.qx[px] = s;
    }
    bank_flush(B, s_cnt, s_status);
}

template <int kFl>
__global__ void __launch_bounds__(kBankBlock) k_bank_collide(const EvTables V, const EvArgs A, const BankArgs B)
{
    __shared__ uint32_t s_cnt[cnt_words(kBankBlock)];
    __shared__ int s_status, s_go;
    const volatile BankCtl *vc = B.ctl;
    if (threadIdx.x == 0) {
        s_status = 0;
        s_go = !(vc->done || vc->status);   // one decision for the whole block
    }
    __syncthreads();
    if (!s_go) return;
    Ctx C;
    // histories that end here fold into the block's shared sums first
    extern __shared__ double s_sums[];
    double *sums = A.smem_sums ? s_sums : nullptr;
    if (sums) {
        for (long long b = threadIdx.x; b < 2 * V.n_bins; b += blockDim.x) sums[b] = 0.0;
        __syncthreads();
    }
    bank_ctx(C, V, A, s_cnt, &s_status, sums);
    const int nc = vc->n_coll;
    // the warp's lanes step through the queue together, so that the
    // free-gas target sampling can share the work across the warp
    for (int j0 = blockIdx.x * blockDim.x; j0 < nc; j0 += gridDim.x * blockDim.x) {
        const int j = j0 + threadIdx.x;
        const bool act = j < nc;
        const int s = act ? B.qc[j] : 0;
        PState p;
        Rng32 R;
        R.init(0u, 0u, 0u, 0u, 0u);
        FgState g;
        int cst = 0;
        if (act) {
            bank_load(B, V, s, p);
            const float4 x = B.fx[s];
            const int2 l = B.fl[s];
            R.init(A.seed, B.hidx[p.hslot], p.id, p.ev, 1u);
            R.prime();   // the event's first block, inline (the collision draws from it)
            Flight f;
            f.sig = x.x;
            f.ss = x.y;
            f.sc = x.z;
            f.xa = XsAt{V.cell_mat[p.cell], l.x, x.w};
            cst = event_collide_begin<kFl>(C, V, R, p, f, g);
        }
        float Vt = 0.f, mu = 0.f;
        if constexpr (kFl != FL_MG && kFl != FL_MGB) {   // multigroup scatters sample no target
            if (!warp_free_gas(C, cst == 2, R, g, Vt, mu) && cst == 2) {
                atomicCAS(&s_status, 0, DS_TIMEOUT);
                cst = 1;
            }
        }
        bool alive = false;
        if (act) {
            alive = cst != 0 && event_collide_end(C, R, p, cst, g, Vt, mu);
            if (alive) {
                B.pw[s] = make_float4(p.x, p.y, p.z, p.wt);
                B.dE[s] = make_float4(p.u, p.v, p.w, p.E);
                if (is_mg<kFl>(V)) B.meta[s] = make_int4(p.cell, p.surf, p.g, p.hslot);
            }
        }
        bank_retire<kFl>(C, B, act && !alive, s, act ? p.hslot : 0);
    }
    bank_flush(B, s_cnt, s_status, &A, sums, V.n_bins);
}

template <int kFl>
__global__ void __launch_bounds__(kBankBlock) k_bank_cross(const EvTables V, const EvArgs A, const BankArgs B)
{
    __shared__ uint32_t s_cnt[cnt_words(kBankBlock)];
    __shared__ int s_status, s_go;
    const volatile BankCtl *vc = B.ctl;
    if (threadIdx.x == 0) {
        s_status = 0;
        s_go = !(vc->done || vc->status);   // one decision for the whole block
    }
    __syncthreads();
    if (!s_go) return;
    Ctx C;
    // histories that end here fold into the block's shared sums first
    extern __shared__ double s_sums[];
    double *sums = A.smem_sums ? s_sums : nullptr;
    if (sums) {
        for (long long b = threadIdx.x; b < 2 * V.n_bins; b += blockDim.x) sums[b] = 0.0;
        __syncthreads();
    }
    bank_ctx(C, V, A, s_cnt, &s_status, sums);
    const int nx = vc->n_cross;
    // split copies wait on the HBM stack; each holds its history open
    auto push = [&](const PState &q, uint32_t cid) -> bool {
        const int k = atomicAdd(&B.ctl->n_split, 1);
        if (k >= B.split_cap) {
            atomicSub(&B.ctl->n_split, 1);
            return false;
        }
        OvfP o;
        o.x = q.x; o.y = q.y; o.z = q.z; o.u = q.u; o.v = q.v; o.w = q.w;
        o.E = q.E; o.wt = q.wt; o.t = q.t; o.cell = q.cell; o.surf = q.surf;
        o.hslot = q.hslot; o.g = q.g;
        o.id = cid;
        B.split[k] = o;
        atomicAdd(&B.hlive[q.hslot], 1);
        return true;
    };
    for (int j0 = blockIdx.x * blockDim.x; j0 < nx; j0 += gridDim.x * blockDim.x) {
        const int j = j0 + threadIdx.x;
        const bool act = j < nx;
        const int s = act ? B.qx[j] : 0;
        PState p;
        bool alive = false;
        if (act) {
            bank_load(B, V, s, p);
            const int2 l = B.fl[s];
            Rng32 R;
            R.init(A.seed, B.hidx[p.hslot], p.id, p.ev, 1u);
            Flight f;
            f.S = l.y >> 2;
            f.sense = (l.y & 3) - 1;
            alive = event_cross<kFl>(C, V, R, p, f, push);
            if (alive) bank_store(B, V, s, p);
        }
        bank_retire<kFl>(C, B, act && !alive, s, act ? p.hslot : 0);
    }
    bank_flush(B, s_cnt, s_status, &A, sums, V.n_bins);
    // the last block to finish closes the iteration
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(&B.ctl->blocks_done, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            volatile BankCtl *c = B.ctl;
            c->n_coll = 0;
            c->n_cross = 0;
            c->iter = c->iter + 1u;
            if (c->n_live == 0 && c->n_split <= 0 && c->next >= A.n) c->done = 1;
            c->blocks_done = 0u;
            __threadfence();
        }
    }
}

__global__ void k_bank_init(BankArgs B)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.P; i += gridDim.x * blockDim.x) {
        B.live[i] = 0;
        B.hlive[i] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        BankCtl c{};
        *B.ctl = c;
    }
}

struct BankKernels {
    void (*adv)(const EvTables, const EvArgs, const BankArgs);
    void (*col)(const EvTables, const EvArgs, const BankArgs);
    void (*crs)(const EvTables, const EvArgs, const BankArgs);
};

BankKernels bank_kernels(int flavor)
{
    if (flavor == FL_CE) return {k_bank_advance<FL_CE>, k_bank_collide<FL_CE>, k_bank_cross<FL_CE>};
    if (flavor == FL_MG) return {k_bank_advance<FL_MGB>, k_bank_collide<FL_MGB>, k_bank_cross<FL_MGB>};
    return {k_bank_advance<FL_ALL>, k_bank_collide<FL_ALL>, k_bank_cross<FL_ALL>};
}

}  // namespace

// Device buffers of the engine; grow only.
struct BankState {
    DevBuf state, rows, mask, ctl, bcnt, split;
    int P = 0;
    long long row_nb = 0;
    bool rows_dirty = true;
};

void bank_state_free(BankState *b)
{
    if (!b) return;
    devbuf_free(b->state);
    devbuf_free(b->rows);
    devbuf_free(b->mask);
    devbuf_free(b->ctl);
    devbuf_free(b->bcnt);
    devbuf_free(b->split);
    delete b;
}

mc_status run_bank(DeviceProblem &d, const EvTables &V, int flavor, bool may_split, uint64_t first, uint64_t n,
                   uint64_t seed, const mc_tune *tune, std::string &err)
{
    if (!d.bank_state) d.bank_state = new BankState();
    BankState &S = *d.bank_state;
    const int P = (tune && tune->bank_capacity) ? (int)tune->bank_capacity : kBankDefault;
    if (P < 1024 || P > (1 << 24) || P % 256 != 0) {
        err = "bank_capacity (the event-split engine's particle slots) must be a multiple of 256 in 1024..2^24";
        return MC_ERR_ARG;
    }
    const long long nb = std::max<long long>(V.n_bins, 1);
    const int nw = (int)((nb + 63) / 64);
    const BankKernels K = bank_kernels(flavor);
    int per_sm = 0, per_sm_c = 0, per_sm_x = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K.adv, kBankBlock, 0);
    const size_t occ_smem = (V.n_bins > 0 && V.n_bins <= 1024) ? 2 * (size_t)V.n_bins * sizeof(double) : 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c, K.col, kBankBlock, occ_smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_x, K.crs, kBankBlock, occ_smem);
    if (per_sm < 1 || per_sm_c < 1 || per_sm_x < 1) { err = "event-split kernels do not fit on an SM"; return MC_ERR_CUDA; }
    const int grid_a = (tune && tune->grid_blocks) ? (int)tune->grid_blocks : d.sms * per_sm;
    const int grid_c = (tune && tune->grid_blocks) ? (int)tune->grid_blocks : d.sms * per_sm_c;
    const int grid_x = (tune && tune->grid_blocks) ? (int)tune->grid_blocks : d.sms * per_sm_x;
    const int grid_max = std::max(grid_a, std::max(grid_c, grid_x));
    // split copies the stack holds: stack_depth when given (a small stack
    // exercises the overflow status), else a quarter of the slots
    const int split_cap = (tune && tune->stack_depth) ? (int)tune->stack_depth : std::max(4096, P / 4);
    if (split_cap < 1 || split_cap > (1 << 24)) {
        err = "stack_depth (the event-split engine's split stack) must be 1..2^24";
        return MC_ERR_ARG;
    }

    // one allocation for the bank's arrays, 256-byte aligned sections
    const size_t Pz = (size_t)P;
    const size_t sizes[] = {16 * Pz, 16 * Pz, 16 * Pz, 8 * Pz, 4 * Pz, 16 * Pz, 8 * Pz,
                            4 * Pz, 4 * Pz, 4 * Pz, 8 * Pz, 4 * Pz};
    size_t total = 0;
    for (size_t z : sizes) total += (z + 255) & ~(size_t)255;
    const size_t row_bytes = Pz * (size_t)nb * sizeof(double);
    const size_t mask_bytes = Pz * (size_t)nw * sizeof(unsigned long long);
    const bool grow_rows = !S.rows.ptr || S.rows.bytes < row_bytes || S.mask.bytes < mask_bytes;
    if (!devbuf_reserve(S.state, total) || !devbuf_reserve(S.rows, row_bytes) ||
        !devbuf_reserve(S.mask, mask_bytes) || !devbuf_reserve(S.ctl, sizeof(BankCtl)) ||
        !devbuf_reserve(S.bcnt, (size_t)grid_max * kNumCounters * sizeof(unsigned long long)) ||
        !devbuf_reserve(S.split, (size_t)split_cap * sizeof(OvfP))) {
        err = "cannot allocate the event-split engine's particle bank";
        return MC_ERR_NOMEM;
    }
    if (grow_rows || S.rows_dirty) {
        cudaMemsetAsync(S.rows.ptr, 0, S.rows.bytes, d.stream);
        cudaMemsetAsync(S.mask.ptr, 0, S.mask.bytes, d.stream);
        S.rows_dirty = false;
    }
    cudaMemsetAsync(S.bcnt.ptr, 0, (size_t)grid_max * kNumCounters * sizeof(unsigned long long), d.stream);
    char *b = static_cast<char *>(S.state.ptr);
    size_t off = 0;
    auto take = [&](size_t z) { char *q = b + off; off += (z + 255) & ~(size_t)255; return q; };
    BankArgs B{};
    B.pw = reinterpret_cast<float4 *>(take(sizes[0]));
    B.dE = reinterpret_cast<float4 *>(take(sizes[1]));
    B.meta = reinterpret_cast<int4 *>(take(sizes[2]));
    B.idev = reinterpret_cast<uint2 *>(take(sizes[3]));
    B.t = reinterpret_cast<float *>(take(sizes[4]));
    B.fx = reinterpret_cast<float4 *>(take(sizes[5]));
    B.fl = reinterpret_cast<int2 *>(take(sizes[6]));
    B.live = reinterpret_cast<int *>(take(sizes[7]));
    B.qc = reinterpret_cast<int *>(take(sizes[8]));
    B.qx = reinterpret_cast<int *>(take(sizes[9]));
    B.hidx = reinterpret_cast<unsigned long long *>(take(sizes[10]));
    B.hlive = reinterpret_cast<int *>(take(sizes[11]));
    B.split = static_cast<OvfP *>(S.split.ptr);
    B.split_cap = split_cap;
    B.P = P;
    B.ctl = static_cast<BankCtl *>(S.ctl.ptr);
    B.bcnt = static_cast<unsigned long long *>(S.bcnt.ptr);
    B.may_split = may_split ? 1 : 0;

    EvArgs A{};
    A.first = first;
    A.n = n;
    A.seed = seed;
    A.max_events = (tune && tune->max_events) ? tune->max_events : kMaxEvents;
    A.acc = static_cast<double *>(S.rows.ptr);
    A.mask = static_cast<unsigned long long *>(S.mask.ptr);
    A.nw = nw;
    A.row_nb = (int)nb;
    A.sum = d.d_sum;
    A.sq = d.d_sq;
    A.tile = 0;          // tally row = the history's slot
    // the collide and cross kernels fold ending histories into per-block
    // shared sums (one global atomic per nonzero bin and block) when the
    // problem has at most 1024 bins; else straight into the global sums
    const bool smem_sums = V.n_bins > 0 && V.n_bins <= 1024;
    const size_t sum_smem = smem_sums ? 2 * (size_t)V.n_bins * sizeof(double) : 0;
    A.smem_sums = smem_sums ? 1 : 0;
    A.n_prob = 0;

    cudaError_t e;
    cudaEventRecord(d.ev[0], d.stream);
    k_bank_init<<<std::max(1, std::min(d.sms * 4, (P + 255) / 256)), 256, 0, d.stream>>>(B);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = cuda_msg(e, "event-split init"); return MC_ERR_CUDA; }
    BankCtl h{};
    uint32_t launches = 1;
    // every particle takes at most max_events events and the bank holds P
    // particles, so the iterations are bounded; the guard only ends a run
    // whose control words went wrong
    const uint64_t iter_cap = (uint64_t)A.max_events * 4 + (n / (uint64_t)P + 1) * (uint64_t)A.max_events;
    uint64_t iters = 0;
    for (;;) {
        for (int k = 0; k < kIterPerCheck; ++k) {
            K.adv<<<grid_a, kBankBlock, 0, d.stream>>>(V, A, B);
            K.col<<<grid_c, kBankBlock, sum_smem, d.stream>>>(V, A, B);
            K.crs<<<grid_x, kBankBlock, sum_smem, d.stream>>>(V, A, B);
        }
        launches += 3 * kIterPerCheck;
        iters += kIterPerCheck;
        if ((e = cudaGetLastError()) != cudaSuccess) { err = cuda_msg(e, "event-split launch"); S.rows_dirty = true; return MC_ERR_CUDA; }
        if ((e = cudaMemcpyAsync(&h, B.ctl, sizeof(h), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
            err = cuda_msg(e, "event-split kernels");
            S.rows_dirty = true;
            return MC_ERR_CUDA;
        }
        if (h.done || h.status) break;
        if (iters > iter_cap) {
            S.rows_dirty = true;
            err = "event-split engine: the iteration bound was reached before every history ended";
            return MC_ERR_TIMEOUT;
        }
    }
    cudaEventRecord(d.ev[1], d.stream);
    std::vector<unsigned long long> bc((size_t)grid_max * kNumCounters);
    if ((e = cudaMemcpyAsync(bc.data(), B.bcnt, bc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        err = cuda_msg(e, "event-split counters");
        S.rows_dirty = true;
        return MC_ERR_CUDA;
    }
    if (h.status != DS_OK) {
        S.rows_dirty = true;
        err = std::string("event-split engine: ") + device_status_text(h.status);
        return status_from_device(h.status);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, d.ev[0], d.ev[1]);
    unsigned long long cnt[kNumCounters] = {};
    for (size_t i = 0; i < bc.size(); ++i) cnt[i % kNumCounters] += bc[i];
    mc_counters &C = d.last;
    std::memset(&C, 0, sizeof(C));
    C.flights = cnt[0]; C.collisions = cnt[1]; C.crossings = cnt[2]; C.tally_updates = cnt[3];
    C.particles = cnt[4]; C.splits = cnt[5]; C.xs_evals = cnt[6]; C.freegas_iters = cnt[7];
    C.nuc_lookups = cnt[8];
    C.histories = n;
    C.transport_ms = ms;
    C.total_ms = ms;
    C.launches = launches;
    d.histories += n;
    d.ntrack += C.flights;
    d.exact_valid = false;   // the mixed mode keeps no per-history rows to sum exactly
    return MC_OK;
}

}  // namespace mc
