// mc_event_kernels.cuh -- device side of the mixed-precision engine: the
// event functions shared by both kernels, the tile kernel (k_event) and the
// per-thread kernel (k_track).  Included by mc_event.cu (host side and the
// tile kernel) and by one translation unit per per-thread kernel flavour
// (mc_event_ce.cu, mc_event_mg.cu, mc_event_all.cu), so that the flavours
// compile in parallel.
#pragma once

#include <cfloat>
#include <cstdint>

#include "mc_engine.h"
#include "mc_evtables.h"
#include "mc_math.cuh"

namespace mc {
namespace ev {   // types the engine's translation units share

// one particle between phases: split copies wait here (overflow bank, HBM)
struct OvfP {
    float x, y, z, u, v, w, E, wt, t;
    int cell, surf, hslot, g;
    uint32_t id;
};

struct EvArgs {
    uint64_t first, n, seed;
    uint32_t max_events;          // events per particle before DS_TIMEOUT
    unsigned long long *next;     // histories handed out (relative)
    double *acc;                  // [grid * tile][row_nb]
    unsigned long long *mask;     // [grid * tile][nw]
    int nw;
    int row_nb;                   // bins per history row (largest problem)
    OvfP *ovf;                    // [grid][ovf_cap]
    int ovf_cap;
    double *sum, *sq;             // global tallies (single problem)
    unsigned long long *counters;
    int *status;
    int tile;
    int smem_sums;                // per-CTA sums live in shared memory
    int refill_min;               // k_track: idle lanes a warp gathers before it starts histories
    // batch of problems (kBatch): history index space = concatenation of
    // every problem's histories
    const EvTables *tabs;         // [n_prob]
    const unsigned long long *prefix;  // [n_prob + 1]
    const unsigned long long *seeds;   // [n_prob]
    double *const *psum;          // [n_prob] per-problem tallies
    double *const *psq;
    int n_prob;
    // batches, and single problems whose sums do not fit in shared memory,
    // fold histories into n_rep > 0 replicas of their bins ([n_rep]
    // [rep_stride], problem p's bins from rep_off[p] on), each CTA into
    // replica blockIdx % n_rep; k_batch_reduce adds them to psum / psq
    double *rsum, *rsq;
    const long long *rep_off;     // [n_prob + 1]
    long long rep_stride;
    int n_rep;
};

enum TileArray {
    TA_X, TA_Y, TA_Z, TA_U, TA_V, TA_W, TA_E, TA_WT, TA_T, TA_SIG, TA_FRAC, TA_SS, TA_SC,
    TA_CELL, TA_SURF, TA_HS, TA_G, TA_GI, TA_SENSE, TA_PROB, TA_XI,
    TA_B0, TA_B1, TA_B2, TA_B3,          // Philox block 0 of the current event
    TA_ID, TA_EV, TA_LIVE, TA_HFREE, TA_HPROB,
    TA_COUNT
};

// Kernel flavours: what code a per-thread kernel carries.  A kernel built
// for one kind of problem leaves out the rest, which would otherwise cost the
// hot loop registers and instruction-cache room.
//   FL_ALL  everything: continuous-energy and multigroup physics, the
//           general scoring path for time filters (one flight may cover
//           several bins, through a pair list in local memory) and the
//           particle comb;
//   FL_CE   continuous energy, no time filter;
//   FL_MG   multigroup, no time filter;
//   FL_MGB  multigroup, no time filter, every tally through the history row
//           (the event-split kernels: nothing stays in a thread's registers
//           from one event kernel to the next).
enum Flavor { FL_ALL = 0, FL_CE = 1, FL_MG = 2, FL_MGB = 3 };

// 128 threads per CTA lets the register budget step through 128 / 80 / 72 /
// 64 registers (4 / 6 / 7 / 8 CTAs per SM)
constexpr int kTrackBlock = 128;
constexpr int kTrackDepth = 32;   // default split copies a thread keeps pending

typedef void (*EvKernel)(const EvTables, const EvArgs);

// the per-thread kernel for (CTAs per SM, batch) in each flavour, one
// translation unit each
EvKernel pick_track_ce(int minb, bool batch);
EvKernel pick_track_mg(int minb, bool batch);
EvKernel pick_track_all(int minb, bool batch);

}  // namespace ev

namespace {
using namespace ev;

constexpr float k2PiF = 6.28318530717959f;
constexpr float kPiHalfF = 1.57079632679490f;
constexpr float kSqrtPiF = 1.77245385090552f;
constexpr float kEpsF = FLT_EPSILON;
constexpr float kInf = __builtin_huge_valf();
constexpr int kMaxFilt = 8;
constexpr int kMaxIl = 32;
constexpr uint32_t kMaxEvents = 1u << 22;   // default events of one particle before MC_ERR_TIMEOUT

enum { C_FLIGHTS = 0, C_COLL, C_CROSS, C_TALLY, C_PART, C_SPLIT, C_XS, C_FREEGAS, C_NUC };



// A 23-bit uniform in (0, 1) from the bits of a block that the four word
// draws leave unused: the low 9 bits of words 0 and 1 and 5 of word 2.
__device__ __forceinline__ float u01f_spare(const U4 &b)
{
    const uint32_t v = (b.x & 0x1FFu) | ((b.y & 0x1FFu) << 9) | ((b.z & 0x1Fu) << 18);
    return ((float)v + 0.5f) * 0x1p-23f;
}

// Where a draw needs a Philox block the stream does not hold yet.  With
// MC_EV_RNG_OUTLINE (the multigroup flavour's translation unit defines it)
// the event's first block is made inline at the start of the flight
// (prime()) and every other refill calls one shared out-of-line copy: such
// refills are rare at run time (most events draw no more than the first
// block's five uniforms), and one copy keeps a full unrolled Philox out of
// every draw site.  Measured on the multigroup slabs: +11 % (30-group deep
// slab) and +15 % (16-layer slab); on the continuous-energy shield the same
// change cost 4 %, so the other flavours keep the refill inline at each
// site.  The random stream is the same either way.
#ifndef MC_EV_RNG_OUTLINE
#define MC_EV_RNG_OUTLINE 0
#endif
#if MC_EV_RNG_OUTLINE
__device__ __noinline__ U4 philox_refill(uint32_t b, uint32_t ev, uint32_t id, uint32_t hlo, uint32_t k0,
                                         uint32_t k1)
{
    return philox(b | 0x80000000u, ev, id, hlo, k0, k1);
}
#endif

// Philox stream of one particle and event, FP32 draws: five 23-bit uniforms
// per block (one per word from its high 23 bits, the fifth from spare low bits)
struct Rng32 {
    uint32_t k0, k1, hlo, id, ev, draw, cached;
    U4 blk;
    __device__ __forceinline__ void init(uint64_t seed, uint64_t hist, uint32_t pid, uint32_t event, uint32_t d)
    {
        k0 = (uint32_t)seed;
        k1 = (uint32_t)(seed >> 32) ^ (uint32_t)(hist >> 32);
        hlo = (uint32_t)hist;
        id = pid;
        ev = event;
        draw = d;
        cached = 0;
    }
    // hand in block 0 computed earlier in the same event
    __device__ __forceinline__ void preload(uint32_t a, uint32_t b, uint32_t c, uint32_t d)
    {
        blk = U4{a, b, c, d};
        cached = 1;
    }
    // the block of the next draw, inline (where an event or a history starts)
    __device__ __forceinline__ void prime()
    {
        const uint32_t b = draw / 5u;
        if (cached != b + 1) {
            blk = philox(b | 0x80000000u, ev, id, hlo, k0, k1);
            cached = b + 1;
        }
    }
    __device__ __forceinline__ float next()
    {
        const uint32_t b = draw / 5u;
        if (cached != b + 1) {
#if MC_EV_RNG_OUTLINE
            blk = philox_refill(b, ev, id, hlo, k0, k1);
#else
            blk = philox(b | 0x80000000u, ev, id, hlo, k0, k1);
#endif
            cached = b + 1;
        }
        const uint32_t q = draw - 5u * b;
        ++draw;
        if (q == 4u) return u01f_spare(blk);
        const uint32_t word = q == 0 ? blk.x : (q == 1 ? blk.y : (q == 2 ? blk.z : blk.w));
        return u01f(word);
    }
};


// shared-memory tile (SoA) and per-CTA bookkeeping.  Every array is addressed
// from the dynamic shared-memory base and the tile size P, so the tile costs
// two registers instead of one pointer per array.  Layout (bytes):
//   [hidx: 8P][30 four-byte arrays: 4P each][qc: 2P][qx: 2P][ssum, ssq: 8 nb each]
struct Tile {
    unsigned char *base;
    int P;
    long long nsum;                      // bins of the per-CTA sums (0: none)
    template <typename X> __device__ __forceinline__ X *a4(int k) const
    {
        return reinterpret_cast<X *>(base + 8 * P + 4 * P * k);
    }
    __device__ __forceinline__ float *x() const { return a4<float>(TA_X); }
    __device__ __forceinline__ float *y() const { return a4<float>(TA_Y); }
    __device__ __forceinline__ float *z() const { return a4<float>(TA_Z); }
    __device__ __forceinline__ float *u() const { return a4<float>(TA_U); }
    __device__ __forceinline__ float *v() const { return a4<float>(TA_V); }
    __device__ __forceinline__ float *w() const { return a4<float>(TA_W); }
    __device__ __forceinline__ float *E() const { return a4<float>(TA_E); }
    __device__ __forceinline__ float *wt() const { return a4<float>(TA_WT); }
    __device__ __forceinline__ float *t() const { return a4<float>(TA_T); }
    __device__ __forceinline__ float *sig() const { return a4<float>(TA_SIG); }
    __device__ __forceinline__ float *frac() const { return a4<float>(TA_FRAC); }
    __device__ __forceinline__ float *ss() const { return a4<float>(TA_SS); }
    __device__ __forceinline__ float *sc() const { return a4<float>(TA_SC); }
    __device__ __forceinline__ int *cell() const { return a4<int>(TA_CELL); }
    __device__ __forceinline__ int *surf() const { return a4<int>(TA_SURF); }
    __device__ __forceinline__ int *hs() const { return a4<int>(TA_HS); }
    __device__ __forceinline__ int *g() const { return a4<int>(TA_G); }
    __device__ __forceinline__ int *gi() const { return a4<int>(TA_GI); }
    __device__ __forceinline__ int *sense() const { return a4<int>(TA_SENSE); }
    __device__ __forceinline__ int *prob() const { return a4<int>(TA_PROB); }
    __device__ __forceinline__ int *xi() const { return a4<int>(TA_XI); }
    __device__ __forceinline__ uint32_t *b0() const { return a4<uint32_t>(TA_B0); }
    __device__ __forceinline__ uint32_t *b1() const { return a4<uint32_t>(TA_B1); }
    __device__ __forceinline__ uint32_t *b2() const { return a4<uint32_t>(TA_B2); }
    __device__ __forceinline__ uint32_t *b3() const { return a4<uint32_t>(TA_B3); }
    __device__ __forceinline__ uint32_t *id() const { return a4<uint32_t>(TA_ID); }
    __device__ __forceinline__ uint32_t *ev() const { return a4<uint32_t>(TA_EV); }
    __device__ __forceinline__ int *live() const { return a4<int>(TA_LIVE); }
    __device__ __forceinline__ int *hfree() const { return a4<int>(TA_HFREE); }
    __device__ __forceinline__ int *hprob() const { return a4<int>(TA_HPROB); }
    __device__ __forceinline__ unsigned long long *hidx() const
    {
        return reinterpret_cast<unsigned long long *>(base);
    }
    __device__ __forceinline__ unsigned short *qc() const
    {
        return reinterpret_cast<unsigned short *>(base + 8 * P + 4 * P * TA_COUNT);
    }
    __device__ __forceinline__ unsigned short *qx() const { return qc() + P; }
    __device__ __forceinline__ double *ssum() const
    {
        return reinterpret_cast<double *>(base + 8 * P + 4 * P * TA_COUNT + 4 * P);
    }
    __device__ __forceinline__ double *ssq() const { return ssum() + nsum; }
    // multigroup k_track with per-CTA sums: each thread's running sum and
    // sum of squares of its register bin ([kTrackBlock][2]), then that bin
    __device__ __forceinline__ double *lane_acc() const { return ssq() + nsum; }
    __device__ __forceinline__ int *lane_bin() const { return reinterpret_cast<int *>(lane_acc() + 2 * kTrackBlock); }
};

struct PState {
    float x, y, z, u, v, w, E, wt, t;
    int cell, surf, hslot, g, prob;
    uint32_t id, ev;
};

__device__ __forceinline__ void load_p(const Tile &T, int s, PState &p)
{
    p.x = T.x()[s]; p.y = T.y()[s]; p.z = T.z()[s]; p.u = T.u()[s]; p.v = T.v()[s]; p.w = T.w()[s];
    p.E = T.E()[s]; p.wt = T.wt()[s]; p.t = T.t()[s];
    p.cell = T.cell()[s]; p.surf = T.surf()[s]; p.hslot = T.hs()[s]; p.g = T.g()[s]; p.prob = T.prob()[s];
    p.id = T.id()[s]; p.ev = T.ev()[s];
}

__device__ __forceinline__ void store_p(const Tile &T, int s, const PState &p)
{
    T.x()[s] = p.x; T.y()[s] = p.y; T.z()[s] = p.z; T.u()[s] = p.u; T.v()[s] = p.v; T.w()[s] = p.w;
    T.E()[s] = p.E; T.wt()[s] = p.wt; T.t()[s] = p.t;
    T.cell()[s] = p.cell; T.surf()[s] = p.surf; T.hs()[s] = p.hslot; T.g()[s] = p.g; T.prob()[s] = p.prob;
    T.id()[s] = p.id; T.ev()[s] = p.ev;
}

// Per-thread event counters live in shared memory, one column per thread
// (conflict-free), which keeps nine registers free for the transport itself.
// Threads come in banks of 128: counter k of thread t is word
// [t / 128][k][t % 128], so a 128-thread block keeps 128 columns, not the
// 256 a wider block needs.
constexpr int kCntStride = 128;
__device__ __forceinline__ uint32_t *cnt_column(uint32_t *s_cnt, int t)
{
    return s_cnt + (t / kCntStride) * (kNumCounters * kCntStride) + (t % kCntStride);
}
// words of the counter array of a block of `threads` threads
__host__ __device__ constexpr int cnt_words(int threads) { return (threads + kCntStride - 1) / kCntStride * kNumCounters * kCntStride; }
struct CounterRef {
    uint32_t *p;
    // an increment is one shared-memory atomic whose result nobody waits for,
    // instead of a load, an add and a store
    __device__ __forceinline__ void operator++(int) const { atomicAdd(p, 1u); }
    __device__ __forceinline__ void operator+=(uint32_t v) const { atomicAdd(p, v); }
    __device__ __forceinline__ void operator=(uint32_t v) const { *p = v; }
    __device__ __forceinline__ operator uint32_t() const { return *p; }
};
struct Counters {
    uint32_t *base;               // this thread's column
    __device__ __forceinline__ CounterRef operator[](int k) const { return CounterRef{base + k * kCntStride}; }
};

struct Ctx {
    const EvTables *V;            // tables of the particle being processed
    const EvArgs *A;
    Tile T;
    Counters cnt;                 // spilled to A.counters before they reach 2^30
    bool reg_mask;                // own rows of at most 128 bins: the touched-bin mask is in registers
    unsigned long long tmask, tmask1;   // bins 0-63 / 64-127 the current history touched (reg_mask)
    int cbin;                     // multigroup kernels: the history's first bin, summed in cval
    double cval;
    int *s_status;
    int *s_novf;
    int *s_nlive;
    int *s_nhfree;
};

// ---------------------------------------------------------------------------
// cross sections
// ---------------------------------------------------------------------------
struct XsAt { int m, i; float f; };   // material, global grid index, fraction

// Macroscopic Sigma_t, Sigma_s, Sigma_c of material m at E (XSec.cpp:9-40
// per nuclide, summed on the union grid): the log2 bucket gives the grid
// point at or below the bucket start, one 32-byte load brings the two rows
// around it ({Sigma_t, Sigma_s, Sigma_c, E} each), and a bounded walk fixes
// the rare bracket miss.  Below the grid the first row's values hold, above
// it the last row's (the fraction is clamped), as XSTable::xs does.
struct XsVal { XsAt at; float st, ss, sc; };

__device__ __forceinline__ XsVal xs_eval(const EvTables &V, int m, float E)
{
    const int off = V.mgrid_off[m], L = V.mgrid_len[m];
    const float4 *row = V.xrow + off;
    int b = (int)((__log2f(E) - V.bkt_lo[m]) * V.bkt_inv[m]);
    b = b < 0 ? 0 : (b >= V.bkt_n[m] ? V.bkt_n[m] - 1 : b);
    int i = __ldg(V.bkt + V.bkt_off[m] + b);
    i = i > L - 2 ? L - 2 : i;
    float4 r0 = __ldg(row + i), r1 = __ldg(row + i + 1);
    while (i > 0 && r0.w > E) { --i; r1 = r0; r0 = __ldg(row + i); }
    while (i < L - 2 && r1.w < E) { ++i; r0 = r1; r1 = __ldg(row + i + 1); }
    float f = (E - r0.w) / (r1.w - r0.w);
    f = f < 0.f ? 0.f : (f > 1.f ? 1.f : f);
    XsVal x;
    x.at = XsAt{m, off + i, f};
    x.st = fmaf(f, r1.x - r0.x, r0.x);
    x.ss = fmaf(f, r1.y - r0.y, r0.y);
    x.sc = fmaf(f, r1.z - r0.z, r0.z);
    return x;
}

// one per-nuclide table on the union grid at a located energy
__device__ __forceinline__ float xs_at(const float *tab, const XsAt &a)
{
    const float y0 = __ldg(tab + a.i), y1 = __ldg(tab + a.i + 1);
    return fmaf(a.f, y1 - y0, y0);
}

enum { XT = 0, XS = 1, XC = 2 };

// whether this particle's problem is multigroup, folded at compile time
// where the flavour decides it
template <int kFl>
__device__ __forceinline__ bool is_mg(const EvTables &V)
{
    return (kFl == FL_MG || kFl == FL_MGB) ? true : (kFl == FL_CE ? false : V.G > 0);
}

// macroscopic cross section of cell material at the particle's energy/group
template <int kFl>
__device__ __forceinline__ float macro(Ctx &C, int m, int which, const PState &p)
{
    const EvTables &V = *C.V;
    C.cnt[C_XS]++;
    if (is_mg<kFl>(V)) {
        const int i = m * V.G + p.g;
        return which == XT ? __ldg(V.mg_total + i) : (which == XS ? __ldg(V.mg_scat_tot + i) : __ldg(V.mg_capture + i));
    }
    const XsVal x = xs_eval(V, m, p.E);
    return which == XT ? x.st : (which == XS ? x.ss : x.sc);
}

// ---------------------------------------------------------------------------
// geometry (FP32, coincident-surface aware)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float surface_eval(const EvTables &V, int s, float x, float y, float z)
{
    const float *k = V.surf_coef + 8 * s;
    switch (V.surf_type[s]) {
    case 0: return x - k[0];
    case 1: return y - k[0];
    case 2: return z - k[0];
    case 3: return k[0] * x + k[1] * y + k[2] * z - k[3];
    case 4: { const float a = x - k[0], b = y - k[1], c = z - k[2]; return a * a + b * b + c * c - k[4]; }
    case 5: { const float a = y - k[0], b = z - k[1]; return a * a + b * b - k[3]; }
    case 6: { const float a = x - k[0], b = y - k[1]; return a * a + b * b - k[3]; }  // cylinder_y as the reference evaluates it
    default: { const float a = x - k[0], b = y - k[1]; return a * a + b * b - k[3]; }
    }
}

// a*a + b*b (+ c*c) - r2 with error-free products and sums (Dekker / Knuth)
__device__ __forceinline__ float comp_sumsq(float a, float b, float c, float r2)
{
    const float pa = a * a, ea = fmaf(a, a, -pa);
    const float pb = b * b, eb = fmaf(b, b, -pb);
    const float pc = c * c, ec = fmaf(c, c, -pc);
    float s = pa + pb;
    float bb = s - pa;
    float err = (pa - (s - bb)) + (pb - bb);
    float s2 = s + pc;
    bb = s2 - s;
    err += (s - (s2 - bb)) + (pc - bb);
    float s3 = s2 - r2;
    bb = s3 - s2;
    err += (s2 - (s3 - bb)) + (-r2 - bb);
    return s3 + (err + ea + eb + ec);
}

// smallest positive root of a t^2 + 2 h t + c = 0 (stable form)
__device__ __forceinline__ float quad_root(float a, float h, float c, bool on)
{
    if (fabsf(a) < 1e-12f) return kInf;
    if (on) {                       // c == 0: roots 0 and -2h/a
        const float t = -2.f * h / a;
        return t > 0.f ? t : kInf;
    }
    const float D = h * h - a * c;
    if (D <= 0.f) return kInf;
    const float sq = sqrtf(D);
    const float q = -(h + copysignf(sq, h));
    float t1 = q / a, t2 = (q != 0.f) ? c / q : kInf;
    t1 = t1 > 0.f ? t1 : kInf;
    t2 = t2 > 0.f ? t2 : kInf;
    return fminf(t1, t2);
}

__device__ float surface_distance(const EvTables &V, int s, const PState &p, bool on)
{
    const float *k = V.surf_coef + 8 * s;
    switch (V.surf_type[s]) {
    case 0: case 1: case 2: {
        if (on) return kInf;
        const int ax = V.surf_type[s];
        const float pos = ax == 0 ? p.x : (ax == 1 ? p.y : p.z);
        const float dir = ax == 0 ? p.u : (ax == 1 ? p.v : p.w);
        if (fabsf(dir) > kEpsF) {
            const float d = (k[0] - pos) / dir;
            return d > 0.f ? d : kInf;
        }
        return kInf;
    }
    case 3: {
        if (on) return kInf;
        const float den = k[0] * p.u + k[1] * p.v + k[2] * p.w;
        if (fabsf(den) > kEpsF) {
            const float d = (k[3] - k[0] * p.x - k[1] * p.y - k[2] * p.z) / den;
            return d > 0.f ? d : kInf;
        }
        return kInf;
    }
    case 4: {
        const float dx = p.x - k[0], dy = p.y - k[1], dz = p.z - k[2];
        const float h = dx * p.u + dy * p.v + dz * p.w;
        const float c = on ? 0.f : comp_sumsq(dx, dy, dz, k[4]);
        return quad_root(1.f, h, c, on);
    }
    case 5: {
        const float dy = p.y - k[0], dz = p.z - k[1];
        const float h = dy * p.v + dz * p.w;
        const float c = on ? 0.f : comp_sumsq(dy, dz, 0.f, k[3]);
        return quad_root(1.f - p.u * p.u, h, c, on);
    }
    case 6: {
        const float dx = p.x - k[0], dz = p.z - k[1];
        const float h = dx * p.u + dz * p.w;
        const float c = on ? 0.f : comp_sumsq(dx, dz, 0.f, k[3]);
        return quad_root(1.f - p.v * p.v, h, c, on);
    }
    default: {
        const float dx = p.x - k[0], dy = p.y - k[1];
        const float h = dx * p.u + dy * p.v;
        const float c = on ? 0.f : comp_sumsq(dx, dy, 0.f, k[3]);
        return quad_root(1.f - p.w * p.w, h, c, on);
    }
    }
}

__device__ void surface_reflect(const EvTables &V, int s, PState &p)
{
    const float *k = V.surf_coef + 8 * s;
    switch (V.surf_type[s]) {
    case 0: p.u = -p.u; break;
    case 1: p.v = -p.v; break;
    case 2: p.w = -p.w; break;
    case 3: {
        const float K = k[0] * p.u + k[1] * p.v + k[2] * p.w;
        p.u -= k[4] * K; p.v -= k[5] * K; p.w -= k[6] * K;
        break;
    }
    default: break;   // the reference leaves quadric reflection a no-op (Geometry.cpp:219-222)
    }
}

__device__ __forceinline__ bool cell_contains(const EvTables &V, int c, const PState &p, int S, bool pos_side)
{
    for (int i = V.cell_surf_off[c]; i < V.cell_surf_off[c + 1]; ++i) {
        const int s2 = V.cell_surf[i];
        const int sense = V.cell_sense[i];
        if (s2 == S) {
            if (sense != 0 && ((sense > 0) != pos_side)) return false;
            continue;
        }
        if (surface_eval(V, s2, p.x, p.y, p.z) * (float)sense < 0.f) return false;
    }
    return true;
}

// cell on the far side of surface S (crossed to the positive side if pos)
__device__ int cell_across(const EvTables &V, const PState &p, int S, bool pos)
{
    const int li = 2 * S + (pos ? 1 : 0);
    for (int k = V.nb_off[li]; k < V.nb_off[li + 1]; ++k) {
        const int c = V.nb_cell[k];
        if (cell_contains(V, c, p, S, pos)) return c;
    }
    for (int c = 0; c < V.n_cell; ++c)
        if (cell_contains(V, c, p, S, pos)) return c;
    return -1;
}

// ---------------------------------------------------------------------------
// tallies (FP32 scores, FP64 per-history accumulation)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int bsearch_f(float x, const float *vec, int n)
{
    int left = 0, right = n - 1;
    while (left <= right) {
        const int mid = (left + right) >> 1;
        if (__ldg(vec + mid) < x) left = mid + 1;
        else right = mid - 1;
    }
    return right;
}

struct Il { int bin; float l; };

__device__ int filter_idx_l(const EvTables &V, int f, const PState &p, float t_old, float speed, float l,
                            Il *out, int cap)
{
    const float *grid = V.filt_grid + V.filt_grid_off[f];
    const int glen = V.filt_grid_len[f];
    const int nbin = glen - 1;
    switch (V.filt_kind[f]) {
    case 0: {
        const int b = bsearch_f((float)p.surf, grid, glen) + 1;
        if (b < 0 || b >= V.filt_size[f]) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 1: {
        const int b = bsearch_f((float)p.cell, grid, glen) + 1;
        if (b < 0 || b >= V.filt_size[f]) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 2: {
        const int b = bsearch_f(p.E, grid, glen);
        if (b < 0 || b >= nbin) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 4:
        out[0].bin = p.g; out[0].l = l; return 1;
    default: {
        const int loc1 = bsearch_f(t_old, grid, glen), loc2 = bsearch_f(p.t, grid, glen);
        if (loc1 == loc2) {
            if (loc1 >= 0 && loc1 < nbin) { out[0].bin = loc1; out[0].l = l; return 1; }
            return 0;
        }
        const int num_bin = loc2 - loc1 - 1;
        const int need = (loc1 >= 0) + (num_bin > 0 ? num_bin : 0) + (loc2 < nbin);
        if (need > cap) return -1;
        int n = 0;
        if (loc1 >= 0) { out[n].bin = loc1; out[n].l = (__ldg(grid + loc1 + 1) - t_old) * speed; ++n; }
        for (int i = 1; i <= num_bin; ++i) {
            out[n].bin = loc1 + i; out[n].l = (__ldg(grid + loc1 + i + 1) - __ldg(grid + loc1 + i)) * speed; ++n;
        }
        if (loc2 < nbin) { out[n].bin = loc2; out[n].l = (p.t - __ldg(grid + loc2)) * speed; ++n; }
        return n;
    }
    }
}

// kFl == FL_MG: the first bin a history scores is summed in registers
// (cbin / cval) and never goes through the row: short multigroup histories
// often score one bin only (a leakage or reflection current).
template <int kFl>
__device__ __forceinline__ void tally_add(Ctx &C, int hslot, int bin, double val)
{
    if constexpr (kFl == FL_MG) {
        if (C.cbin == bin || C.cbin < 0) {
            C.cbin = bin;
            C.cval += val;
            C.cnt[C_TALLY]++;
            return;
        }
    }
    // the value and the touched bit are reductions in L2 that the thread does
    // not wait for; rows of at most 128 bins keep the touched bits in registers
    const size_t row = (size_t)blockIdx.x * C.A->tile + hslot;
    atomicAdd(C.A->acc + row * C.A->row_nb + bin, val);
    const unsigned long long bit = 1ull << (bin & 63);
    if (C.reg_mask) {
        if (bin & 64) C.tmask1 |= bit;
        else C.tmask |= bit;
    } else {
        atomicOr(C.A->mask + row * C.A->nw + (bin >> 6), bit);
    }
    C.cnt[C_TALLY]++;
}

template <int kFl>
__device__ float score_value(Ctx &C, int sc, const PState &p, float l)
{
    const EvTables &V = *C.V;
    const int m = V.cell_mat[p.cell];
    const int kern = V.score_kernel[sc], kind = V.score_kind[sc];
    // the cross sections this score needs come from one lookup (one copy of
    // the lookup code per scoring site); a void cell scores zero
    float st = 0.f, ss = 0.f, sc_ = 0.f;
    if (m >= 0 && (kern == 1 || kind != 0)) {
        if (is_mg<kFl>(V)) {
            const int i = m * V.G + p.g;
            st = __ldg(V.mg_total + i);
            ss = __ldg(V.mg_scat_tot + i);
            sc_ = __ldg(V.mg_capture + i);
        } else {
            const XsVal x = xs_eval(V, m, p.E);
            st = x.st;
            ss = x.ss;
            sc_ = x.sc;
        }
        C.cnt[C_XS] += (kern == 1 ? 1u : 0u) + (kind != 0 ? 1u : 0u);
    }
    const float k = kern == 0 ? p.wt * l : (kern == 1 ? p.wt / st : p.wt);
    switch (kind) {
    case 0: return k;
    case 1: case 3: return sc_ * k;
    case 2: return ss * k;
    default: return st * k;
    }
}

// Estimator::score (Estimator.cpp:298-336) for estimators without a time
// filter: every filter yields one (bin, length) pair or none, all lengths
// equal l_in, so the combination loop collapses to one flattened index and
// needs no pair list (which would live in local memory).
//
// pre / fixed: an estimator attached to a cell (track-length, collision) or
// to a surface (crossing) has its cell or surface filter fixed by the
// attachment.  The table builder resolved that filter's part of the flattened
// index once per attachment (pre; -1: the cell or surface lies outside the
// filter, nothing is scored), and the loop skips filters of kind `fixed`.
template <int kFl>
__device__ __forceinline__ bool estimator_score_simple(Ctx &C, int e, const PState &p, float l_in, int pre,
                                                       int fixed)
{
    const EvTables &V = *C.V;
    const int f0 = V.est_filt_off[e], nf = V.est_filt_off[e + 1] - f0;
    const int *fac = V.est_factor + V.est_factor_off[e];
    if (pre < 0) return true;
    int idx1 = pre;
    for (int i = 0; i < nf; ++i) {
        const int f = f0 + i;
        const int kind = V.filt_kind[f];
        if (kind == fixed) continue;
        const float *grid = V.filt_grid + V.filt_grid_off[f];
        const int glen = V.filt_grid_len[f];
        int b;
        switch (kind) {
        case 0: b = bsearch_f((float)p.surf, grid, glen) + 1; if (b < 0 || b >= V.filt_size[f]) return true; break;
        case 1: b = bsearch_f((float)p.cell, grid, glen) + 1; if (b < 0 || b >= V.filt_size[f]) return true; break;
        case 2: b = bsearch_f(p.E, grid, glen); if (b < 0 || b >= glen - 1) return true; break;
        case 4: b = p.g; break;
        default: return false;          // time filter: take the general path
        }
        idx1 += b * fac[i + 1];
    }
    const int s0 = V.est_score_off[e], ns = V.est_score_off[e + 1] - s0;
    const int base = V.est_bin_off[e];
    for (int s = 0; s < ns; ++s) {
        tally_add<kFl>(C, p.hslot, base + idx1, (double)score_value<kFl>(C, s0 + s, p, l_in));
        idx1 += fac[0];
    }
    return true;
}


// Estimator::score (Estimator.cpp:298-336).  pre / fixed as for
// estimator_score_simple; the general path recomputes every filter.
template <int kFl>
__device__ void estimator_score(Ctx &C, int e, const PState &p, float t_old, float speed, float l_in, int pre,
                                int fixed)
{
    const EvTables &V = *C.V;
    if (!(fabsf(l_in) <= FLT_MAX)) {   // non-finite track: the loop below would never advance
        atomicCAS(C.s_status, 0, DS_NAN);
        return;
    }
    if (estimator_score_simple<kFl>(C, e, p, l_in, pre, fixed)) return;
    if constexpr (kFl != FL_ALL) {
        atomicCAS(C.s_status, 0, DS_OVERFLOW);   // unreachable: time filters get the FL_ALL kernel
        return;
    }
    const int f0 = V.est_filt_off[e], nf = V.est_filt_off[e + 1] - f0;
    const int s0 = V.est_score_off[e], ns = V.est_score_off[e + 1] - s0;
    const int *fac = V.est_factor + V.est_factor_off[e];
    const int base = V.est_bin_off[e];
    if (!(fabsf(l_in) <= FLT_MAX)) {   // non-finite track: the loop below would never advance
        atomicCAS(C.s_status, 0, DS_NAN);
        return;
    }
    Il il[kMaxIl];
    int off[kMaxFilt + 1], nil[kMaxFilt], idx[kMaxFilt];
    off[0] = 0;
    for (int i = 0; i < nf; ++i) {
        const int n = filter_idx_l(V, f0 + i, p, t_old, speed, l_in, il + off[i], kMaxIl - off[i]);
        if (n < 0) { atomicCAS(C.s_status, 0, DS_OVERFLOW); return; }
        if (n == 0) return;
        nil[i] = n;
        off[i + 1] = off[i] + n;
        idx[i] = 0;
    }
    for (int guard = 0; guard <= off[nf]; ++guard) {   // each pass advances one filter
        float l = FLT_MAX;
        for (int i = 0; i < nf; ++i) { const float x = il[off[i] + idx[i]].l; l = (x < l) ? x : l; }
        int idx1 = 0;
        for (int i = 0; i < nf; ++i) idx1 += il[off[i] + idx[i]].bin * fac[i + 1];
        for (int s = 0; s < ns; ++s) {
            tally_add<FL_ALL>(C, p.hslot, base + idx1, (double)score_value<FL_ALL>(C, s0 + s, p, l));
            idx1 += fac[0];
        }
        for (int i = 0; i < nf; ++i) {
            Il &cur = il[off[i] + idx[i]];
            cur.l -= l;
            if (cur.l < kEpsF) {
                if (idx[i] == nil[i] - 1) return;
                idx[i]++;
            }
        }
        if (nf == 0) return;
    }
}

// ---------------------------------------------------------------------------
// particle life cycle
// ---------------------------------------------------------------------------
// Folds a finished history's row into the sums (Estimator.cpp:339-346):
// per-CTA shared sums for one problem, the problem's global sums in a batch.
template <int kFl, bool kPair>
__device__ void history_fold(Ctx &C, int hslot, int prob)
{
    const size_t row = (size_t)blockIdx.x * C.A->tile + hslot;
    double *acc = C.A->acc + row * C.A->row_nb;
    unsigned long long *mask = C.A->mask + row * C.A->nw;
    double *gs = C.A->sum, *gq = C.A->sq;
    if (C.A->n_rep > 0) {
        // this CTA's replica of the problem's bins.  Histories of one
        // problem fold at the same time all over the GPU; into one set of
        // sums their FP64 additions to the same few addresses queue up at
        // L2 (a batch: about 10^9 histories/s in all, whatever the problem)
        const size_t at = (size_t)(blockIdx.x % C.A->n_rep) * (size_t)C.A->rep_stride +
                          (size_t)(C.A->n_prob > 0 ? C.A->rep_off[prob] : 0);
        gs = C.A->rsum + at;
        gq = C.A->rsq + at;
    }
    if constexpr (kFl == FL_MG) {
        if (C.cbin >= 0) {
            const double v = C.cval;
            if (C.A->smem_sums) {
                // the thread's own running sums of the bin (no other thread
                // touches them; most of a thread's histories score the same
                // bin): the CTA's sums take a pair of shared-memory atomics
                // when the bin changes, not one per history
                double *la = C.T.lane_acc() + 2 * threadIdx.x;
                int *lb = C.T.lane_bin() + threadIdx.x;
                if (*lb == C.cbin) {
                    la[0] += v;
                    la[1] += v * v;
                } else {
                    if (*lb >= 0) {
                        atomicAdd(C.T.ssum() + *lb, la[0]);
                        atomicAdd(C.T.ssq() + *lb, la[1]);
                    }
                    *lb = C.cbin;
                    la[0] = v;
                    la[1] = v * v;
                }
            } else {
                atomicAdd(gs + C.cbin, v);
                atomicAdd(gq + C.cbin, v * v);
            }
            C.cbin = -1;
            C.cval = 0.0;
        }
    }
    for (int wi = 0; wi < C.A->nw; ++wi) {
        unsigned long long m;
        if (C.reg_mask) {   // nw <= 2
            m = wi == 0 ? C.tmask : C.tmask1;
            if (m == 0ull) continue;
        } else {
            if (__ldcg(mask + wi) == 0ull) continue;
            m = atomicExch(mask + wi, 0ull);
        }
        // the row holds reductions: read and clear each touched bin in L2
        auto take = [&](int bin) {
            return __longlong_as_double(
                (long long)atomicExch(reinterpret_cast<unsigned long long *>(acc + bin), 0ull));
        };
        auto add = [&](int bin, double v) {
            if (C.A->smem_sums) {
                atomicAdd(C.T.ssum() + bin, v);
                atomicAdd(C.T.ssq() + bin, v * v);
            } else {
                atomicAdd(gs + bin, v);
                atomicAdd(gq + bin, v * v);
            }
        };
        while (m) {
            const int b0 = wi * 64 + __ffsll((long long)m) - 1;
            m &= m - 1;
            const double v0 = take(b0);
            if (kPair && m) {
                // two exchanges in flight before either value is used: half
                // the L2 round trips in sequence (measured +10 % on a
                // 30-group slab; in the batch kernel the extra live
                // registers cost more than the latency saved)
                const int b1 = wi * 64 + __ffsll((long long)m) - 1;
                m &= m - 1;
                const double v1 = take(b1);
                add(b0, v0);
                add(b1, v1);
            } else {
                add(b0, v0);
            }
        }
    }
    C.tmask = 0ull;
    C.tmask1 = 0ull;
    C.cbin = -1;
    C.cval = 0.0;
}

__device__ __forceinline__ void particle_dies(Ctx &C, int s, int hslot)
{
    C.T.hs()[s] = -1;
    atomicSub(C.s_nlive, 1);
    if (atomicSub(&C.T.live()[hslot], 1) == 1) {
        __threadfence_block();
        history_fold<FL_ALL, false>(C, hslot, C.T.hprob()[hslot]);
        const int k = atomicAdd(C.s_nhfree, 1);
        C.T.hfree()[k] = hslot;
    }
}

__device__ __forceinline__ float speed_of(float E) { return 1383159.26439f * sqrtf(E); }

// Algorithm.cpp:67-101 in FP32
__device__ __forceinline__ void scatter_direction(Rng32 &R, float dx, float dy, float dz, float mu0,
                                                  float &ox, float &oy, float &oz)
{
    float sa, ca;
    __sincosf(k2PiF * R.next(), &sa, &ca);
    const float Ac = sqrtf(fmaxf(1.f - mu0 * mu0, 0.f));
    // the reference swaps to the y axis only for dz == 1 exactly; in FP32 a
    // direction within 0.99 of +-z loses the formula's precision (and dz == -1
    // divides by zero), so the swap covers both poles
    if (fabsf(dz) < 0.99f) {
        const float B = sqrtf(1.f - dz * dz);
        const float Cc = Ac / B;
        ox = dx * mu0 + (dx * dz * ca - dy * sa) * Cc;
        oy = dy * mu0 + (dy * dz * ca + dx * sa) * Cc;
        oz = dz * mu0 - ca * Ac * B;
    } else {
        const float B = sqrtf(fmaxf(1.f - dy * dy, 1e-30f));
        const float Cc = Ac / B;
        ox = dx * mu0 + (dx * dy * ca - dz * sa) * Cc;
        oz = dz * mu0 + (dz * dy * ca + dx * sa) * Cc;
        oy = dy * mu0 - ca * Ac * B;
    }
    const float r = rsqrtf(ox * ox + oy * oy + oz * oz);
    ox *= r; oy *= r; oz *= r;
}

// Free-gas elastic scatter (Reaction.cpp:27-118) in FP32, in three parts so
// that the per-thread kernel can sample the target velocity for a whole warp
// at once.  Candidate k of a scatter draws its six numbers from a Philox
// block of its own (counter word 0xC0000000 | k, disjoint from the event's
// ordinary blocks), as six 21-bit uniforms, so any lane can evaluate any
// particle's k-th candidate and the accepted one does not depend on who
// evaluated it.
struct FgState { float A, mu0, speed, beta, p_g2; };

__device__ __forceinline__ void free_gas_begin(Rng32 &R, const PState &p, float A, FgState &g)
{
    g.A = A;
    g.mu0 = 2.f * R.next() - 1.f;
    g.speed = speed_of(p.E);
    g.beta = sqrtf(2.0659834e-11f * A);
    const float y = g.beta * g.speed;
    g.p_g2 = 2.f / (2.f + kSqrtPiF * y);
}

// Reaction.cpp:48-66: target speed V and cosine mu of candidate k, and
// whether the rejection test accepts it.  Compiled once (noinline), so the
// sequential and the warp-cooperative samplers get the same bits.
__device__ __forceinline__ bool fg_candidate(float speed, float beta, float p_g2, uint32_t k0, uint32_t k1,
                                          uint32_t hlo, uint32_t id, uint32_t ev, uint32_t k, float &V, float &mu)
{
    const U4 a = philox(0xC0000000u | k, ev, id, hlo, k0, k1);
    // six 21-bit uniforms: the high 21 bits of each word, then two from the
    // low bits (11 + 10, and 1 + 11 + 9)
    const float sc = 0x1p-21f;
    const float r0 = ((float)(a.x >> 11) + 0.5f) * sc;
    const float r1 = ((float)(a.y >> 11) + 0.5f) * sc;
    const float r2 = ((float)(a.z >> 11) + 0.5f) * sc;
    const float r3 = ((float)(a.w >> 11) + 0.5f) * sc;
    const float r4 = ((float)((a.x & 0x7FFu) | ((a.y & 0x3FFu) << 11)) + 0.5f) * sc;
    const float r5 = ((float)(((a.y >> 10) & 1u) | ((a.z & 0x7FFu) << 1) | ((a.w & 0x1FFu) << 12)) + 0.5f) * sc;
    // Reaction.cpp:48-57 without the branch: the "w2" form sqrt(-ln(a b)) is
    // the "w1" form sqrt(-ln u1 - ln u2 cos^2) with cos = 1
    const bool w2 = r0 < p_g2;
    const float cv = w2 ? 1.f : __cosf(kPiHalfF * r3);
    const float x = sqrtf(-__logf(r1) - __logf(r2) * (cv * cv));
    V = x / beta;
    mu = 2.f * r4 - 1.f;
    const float acc = sqrtf(fmaxf(speed * speed + V * V - 2.f * speed * V * mu, 0.f)) / (speed + V);
    return !(r5 > acc);
}

constexpr uint32_t kFgMaxCandidates = 1u << 16;

// a / b for 0 <= a <= 64 and 1 <= b <= 32, exactly: (a + 1/2) / b lies at
// least 1/64 from an integer, far more than the rounding of one reciprocal
// and one product (checked for every pair by the test suite's restatement)
__device__ __forceinline__ int div_small(int a, int b)
{
    return (int)__fmul_rn(__fadd_rn((float)a, 0.5f), __frcp_rn((float)b));
}

// position of the n-th (0-based) set bit of m; n < popc(m)
__device__ __forceinline__ int nth_set_bit(unsigned m, int n)
{
    int base = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc((m >> base) & ((1u << w) - 1u));
        if (n >= c) { n -= c; base += w; }
    }
    return base;
}

// The rejection loop for every pending lane of the warp at once; all 32
// lanes must call it.  After the first round (each particle's own first
// candidate), each round every lane evaluates one candidate: lane L works on
// pending particle (L mod np) at offset (L div np) past the candidates that
// particle has already tried.  A particle takes its first
// accepted candidate in candidate order, which is the one the sequential loop
// accepts; a warp needs about two rounds where the sequential loop needs the
// longest rejection chain among its lanes.
__device__ __forceinline__ bool warp_free_gas(Ctx &C, bool pend, const Rng32 &R, const FgState &g, float &V,
                                              float &mu)
{
    const int lane = threadIdx.x & 31;
    uint32_t tried = 0;
    for (uint32_t round = 0;; ++round) {
        const unsigned pm = __ballot_sync(0xffffffffu, pend);
        if (pm == 0u) return true;
        if (round >= kFgMaxCandidates) return !pend;
        // the first round: each pending particle tries its own first
        // candidate in its own lane; later rounds share the lanes among the
        // pending particles
        const int np = __popc(pm);
        int which = 0, off = 0, src = lane;
        float s_speed = g.speed, s_beta = g.beta, s_pg2 = g.p_g2;
        uint32_t s_k0 = R.k0, s_k1 = R.k1, s_hlo = R.hlo, s_id = R.id, s_ev = R.ev, s_tried = 0u;
        if (round > 0) {
            off = div_small(lane, np);
            which = lane - off * np;
            src = nth_set_bit(pm, which);
            s_speed = __shfl_sync(0xffffffffu, g.speed, src);
            s_beta = __shfl_sync(0xffffffffu, g.beta, src);
            s_pg2 = __shfl_sync(0xffffffffu, g.p_g2, src);
            s_k0 = __shfl_sync(0xffffffffu, R.k0, src);
            s_k1 = __shfl_sync(0xffffffffu, R.k1, src);
            s_hlo = __shfl_sync(0xffffffffu, R.hlo, src);
            s_id = __shfl_sync(0xffffffffu, R.id, src);
            s_ev = __shfl_sync(0xffffffffu, R.ev, src);
            s_tried = __shfl_sync(0xffffffffu, tried, src);
        }
        float Vc, muc;
        const bool hit = fg_candidate(s_speed, s_beta, s_pg2, s_k0, s_k1, s_hlo, s_id, s_ev,
                                      s_tried + (uint32_t)off, Vc, muc);
        if (round == 0) {
            if (pend) {
                tried = 1u;
                if (hit) {
                    C.cnt[C_FREEGAS] += 1u;
                    V = Vc;
                    mu = muc;
                    pend = false;
                }
            }
            continue;
        }
        const unsigned sm = __ballot_sync(0xffffffffu, hit);
        int first = -1, r = 0;
        if (pend) {
            r = __popc(pm & ((1u << lane) - 1u));   // this particle's rank among the pending
            for (int L = r; L < 32; L += np)
                if ((sm >> L) & 1u) { first = L; break; }
        }
        const int sel = first >= 0 ? first : lane;
        const float Vs = __shfl_sync(0xffffffffu, Vc, sel);
        const float ms = __shfl_sync(0xffffffffu, muc, sel);
        if (pend) {
            if (first >= 0) {
                tried += (uint32_t)div_small(first, np) + 1u;
                C.cnt[C_FREEGAS] += tried;
                V = Vs;
                mu = ms;
                pend = false;
            } else {
                tried += (uint32_t)div_small(32 - r + np - 1, np);
            }
        }
    }
}

// Reaction.cpp:67-118: the outgoing velocity from the accepted target
// velocity (two scatter_direction draws from the event's stream)
__device__ __forceinline__ void free_gas_finish(Rng32 &R, PState &p, const FgState &g, float V, float mu)
{
    const float A = g.A, speed = g.speed;
    float nx, ny, nz;
    scatter_direction(R, p.u, p.v, p.w, mu, nx, ny, nz);
    const float inv = 1.f / (1.f + A);
    const float ux = (speed * p.u + A * (nx * V)) * inv;
    const float uy = (speed * p.v + A * (ny * V)) * inv;
    const float uz = (speed * p.w + A * (nz * V)) * inv;
    const float cx = speed * p.u - ux, cy = speed * p.v - uy, cz = speed * p.w - uz;
    const float sc = sqrtf(cx * cx + cy * cy + cz * cz);
    const float isc = 1.f / sc;
    float dx, dy, dz;
    scatter_direction(R, cx * isc, cy * isc, cz * isc, g.mu0, dx, dy, dz);
    const float vx = sc * dx + ux, vy = sc * dy + uy, vz = sc * dz + uz;
    const float vs = sqrtf(vx * vx + vy * vy + vz * vz);
    const float ivs = 1.f / vs;
    p.E = 5.2270376e-13f * vs * vs;
    p.u = vx * ivs; p.v = vy * ivs; p.w = vz * ivs;
}

__device__ __forceinline__ void weight_roulette(Ctx &C, Rng32 &R, PState &p, bool &alive)
{
    if (p.wt < C.V->wr) {
        if (R.next() < p.wt / C.V->ws) p.wt = C.V->ws;
        else alive = false;
    }
}

// SourceBank / SourcePoint (Source.cpp:20-24, 42-45), FP32
__device__ void sample_source(const EvTables &V, uint64_t seed, uint64_t hist, PState &p)
{
    Rng32 R;
    R.init(seed, hist, 0u, 0u, 0u);
    R.prime();
    const float xi = R.next();
    int s = bsearch_f(xi, V.src_cdf, V.n_src + 1);
    s = s < 0 ? 0 : (s >= V.n_src ? V.n_src - 1 : s);
    const float *ep = V.src_e_par + 2 * s;
    const float E = (V.src_e_kind[s] == 1) ? ep[0] + R.next() * ep[1] : ep[0];
    const float *dp = V.src_dir_par + 9 * s;
    const int dk = V.src_dir_kind[s];
    float d0, d1, d2;
    if (dk == 0) {
        d0 = dp[0]; d1 = dp[1]; d2 = dp[2];
    } else if (dk == 1 || dk == 3) {
        const float mu = (dk == 1) ? 2.f * R.next() - 1.f : R.next();
        float sa, ca;
        __sincosf(k2PiF * R.next(), &sa, &ca);
        const float c = sqrtf(fmaxf(1.f - mu * mu, 0.f));
        d0 = mu; d1 = ca * c; d2 = sa * c;
    } else {
        float d[3];
        for (int k = 2; k >= 0; --k) {
            const float *q = dp + 3 * k;
            d[k] = ((int)q[0] == 1) ? q[1] + R.next() * q[2] : q[1];
        }
        d0 = d[0]; d1 = d[1]; d2 = d[2];
    }
    p.x = V.src_pos[3 * s]; p.y = V.src_pos[3 * s + 1]; p.z = V.src_pos[3 * s + 2];
    p.u = d0; p.v = d1; p.w = d2;
    p.E = E; p.wt = 1.f; p.t = 0.f;
    p.cell = V.src_cell[s];
    p.surf = -1;
    p.g = V.src_group[s];
    p.id = 0u;
    p.ev = 0u;
    p.prob = 0;
}

// ---------------------------------------------------------------------------
// one event of one particle, shared by both kernels
// ---------------------------------------------------------------------------
// What the advance step hands to the collision or crossing step.
struct Flight {
    float sig;      // Sigma_t at the collision site
    float ss, sc;   // Sigma_s, Sigma_c there (CE)
    XsAt xa;        // its place on the material's union grid (CE)
    int S, sense;   // surface to cross and the cell's sense of it
};

// general.cpp:40-83: cross section, distance to collision (draw 0 of the
// event), nearest surface, flight and track-length tallies.  Returns 1 for a
// collision, 2 for a crossing, 0 if the particle is lost (status set).
template <int kFl>
__device__ __forceinline__ int event_advance(Ctx &C, const EvTables &V, Rng32 &R, PState &p, Flight &f)
{
#if MC_EV_RNG_OUTLINE
    R.prime();   // the event's first Philox block, inline: the event's later draws read it
#endif
    const int m = V.cell_mat[p.cell];
    float dcol;
    f.sig = 0.f;
    f.ss = 0.f;
    f.sc = 0.f;
    f.xa = XsAt{m, 0, 0.f};
    if (m >= 0) {
        if (is_mg<kFl>(V)) {
            f.sig = macro<kFl>(C, m, XT, p);
        } else {
            const XsVal x = xs_eval(V, m, p.E);
            f.xa = x.at;
            f.sig = x.st;
            f.ss = x.ss;
            f.sc = x.sc;
            C.cnt[C_XS]++;
        }
        dcol = -__logf(R.next()) / f.sig;
    } else {
        dcol = 0.9f * FLT_MAX;
    }
    float dist = kInf;
    f.S = -1;
    f.sense = 0;
    for (int i = V.cell_surf_off[p.cell]; i < V.cell_surf_off[p.cell + 1]; ++i) {
        const int sf = V.cell_surf[i];
        const float d = surface_distance(V, sf, p, sf == p.surf);
        if (d < dist) { dist = d; f.S = sf; f.sense = V.cell_sense[i]; }
    }
    const bool cross = dcol > dist;
    if (cross && f.S < 0) {
        atomicCAS(C.s_status, 0, DS_LOST);
        return 0;
    }
    const float l = cross ? dist : dcol;
    const float t_old = p.t;
    p.x = fmaf(p.u, l, p.x); p.y = fmaf(p.v, l, p.y); p.z = fmaf(p.w, l, p.z);
    float speed = 0.f;
    if (V.has_time) {
        speed = speed_of(p.E);
        p.t = t_old + l / speed;
    }
    C.cnt[C_FLIGHTS]++;
    if (m >= 0 && !is_mg<kFl>(V)) C.cnt[C_NUC] += (uint32_t)(V.mnuc_off[m + 1] - V.mnuc_off[m]);
    for (int i = V.cell_tl_off[p.cell]; i < V.cell_tl_off[p.cell + 1]; ++i)
        estimator_score<kFl>(C, V.cell_tl[i], p, t_old, speed, l, V.cell_tl_pre[i], 1);
    p.surf = -1;
    return cross ? 2 : 1;
}

// general.cpp:121-163 and population_control.cpp:9-15 in two halves around
// the free-gas target sampling.  The first half: collision tallies, implicit
// capture, scatter nuclide (or the multigroup transfer); R continues the
// event's stream after the distance draw.  Returns 0 if the particle dies (a
// void cell), 1 if it needs no target sampling, 2 if it scatters on a
// nuclide by free gas (g holds the sampling parameters).
template <int kFl>
__device__ __forceinline__ int event_collide_begin(Ctx &C, const EvTables &V, Rng32 &R, PState &p, const Flight &f,
                                                   FgState &g)
{
    C.cnt[C_COLL]++;
    const int m = V.cell_mat[p.cell];
    if (m < 0) return 0;
    for (int i = V.cell_c_off[p.cell]; i < V.cell_c_off[p.cell + 1]; ++i)
        estimator_score<kFl>(C, V.cell_c[i], p, p.t, V.has_time ? speed_of(p.E) : 0.f, 0.f,
                                       V.cell_c_pre[i], 1);
    const float st = f.sig;
    if (is_mg<kFl>(V)) {
        const int row = m * V.G + p.g;
        p.wt = p.wt * (st - __ldg(V.mg_capture + row)) / st;
        const float *cdf = V.mg_cdf + (size_t)row * V.G;
        const float u = __ldg(cdf + V.G - 1) * R.next();
        // first group whose cumulative row entry exceeds u, by bisection
        // (the same group a linear scan finds: the row is non-decreasing)
        int lo = 0, hi = V.G;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(cdf + mid) > u) hi = mid;
            else lo = mid + 1;
        }
        const int gout = lo < V.G ? lo : -1;
        if (gout >= 0) {
            p.g = gout;
            const float mu = 2.f * R.next() - 1.f;
            float nx, ny, nz;
            scatter_direction(R, p.u, p.v, p.w, mu, nx, ny, nz);
            p.u = nx; p.v = ny; p.w = nz;
        }
        C.cnt[C_XS]++;
        return 1;
    }
    const XsAt &a = f.xa;
    const float sc = f.sc, ss = f.ss;   // from the advance step's rows
    C.cnt[C_XS] += 2;
    p.wt = p.wt * (st - sc) / st;
    const float u = ss * R.next();
    float acc = 0.f;
    int nuc = -1;
    for (int k = V.mnuc_off[m]; k < V.mnuc_off[m + 1]; ++k) {
        acc += xs_at(V.nucS + V.mnuc_tab[k] - V.mgrid_off[m], a);
        if (acc > u) { nuc = V.mnuc_id[k]; break; }
    }
    if (nuc < 0) return 1;   // no scatter nuclide: the reference returns without scattering
    free_gas_begin(R, p, __ldg(V.nuc_A + nuc), g);
    return 2;
}

// The second half: the outgoing velocity of a free-gas scatter (st == 2,
// target velocity V, mu), the finiteness check and weight roulette.
__device__ __forceinline__ bool event_collide_end(Ctx &C, Rng32 &R, PState &p, int st, const FgState &g, float V,
                                                  float mu)
{
    if (st == 2) free_gas_finish(R, p, g, V, mu);
    if (!(fabsf(p.E) <= FLT_MAX && fabsf(p.u) <= 1.5f && fabsf(p.wt) <= FLT_MAX)) {
        atomicCAS(C.s_status, 0, DS_NAN);
        return false;
    }
    bool alive = true;
    weight_roulette(C, R, p, alive);
    return alive;
}

// general.cpp:89-115 and population_control.cpp:21-49: new cell, boundary
// condition, crossing tallies, importance roulette / splitting, weight
// roulette.  R must stand at draw 1 of the event.  Split copies go to
// push(p, id), which returns false when its store is full.
template <int kFl, typename Push>
__device__ __forceinline__ bool event_cross(Ctx &C, const EvTables &V, Rng32 &R, PState &p, const Flight &f,
                                            Push &&push)
{
    C.cnt[C_CROSS]++;
    const int S = f.S;
    const int old_cell = p.cell;
    bool alive = true;
    const int bc = V.surf_bc[S];
    p.surf = S;
    if (bc == 0) {
        const bool pos = !(f.sense > 0);
        const int c = cell_across(V, p, S, pos);
        if (c < 0) { atomicCAS(C.s_status, 0, DS_LOST); alive = false; }
        else p.cell = c;
    } else if (bc == -1) {
        alive = false;
        p.wt = 0.f;
    } else {
        surface_reflect(V, S, p);
    }
    if (p.wt != 0.f) {   // a vacuum boundary kills first and scores zero (general.cpp:98-111)
        const float speed = V.has_time ? speed_of(p.E) : 0.f;
        for (int i = V.surf_est_off[S]; i < V.surf_est_off[S + 1]; ++i)
            estimator_score<kFl>(C, V.surf_est[i], p, p.t, speed, 0.f, V.surf_est_pre[i], 0);
    }
    if (alive && p.cell != old_cell) {
        const float Iold = V.cell_imp[old_cell], Inew = V.cell_imp[p.cell];
        if (Inew != Iold) {
            const float rat = Inew / Iold;
            if (rat < 1.f) {
                if (R.next() < rat) p.wt = p.wt / rat;
                else alive = false;
            } else {
                const int n = (int)floorf(rat + R.next());
                p.wt = p.wt / (float)n;
                for (int k = 1; k < n; ++k) {
                    if (!push(p, child_id(p.id, p.ev, (uint32_t)k))) {
                        atomicCAS(C.s_status, 0, DS_OVERFLOW);
                        break;
                    }
                    C.cnt[C_SPLIT]++;
                }
            }
        }
    }
    if (alive) weight_roulette(C, R, p, alive);
    return alive;
}

// ---------------------------------------------------------------------------
// the persistent kernel
// ---------------------------------------------------------------------------
__device__ __forceinline__ int warp_append(int *counter, bool pred)
{
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (m) {
        const int leader = __ffs(m) - 1;
        if (lane == leader) base = atomicAdd(counter, __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + __popc(m & ((1u << lane) - 1u));
}

// problem of a position in the concatenated history space of a batch
__device__ __forceinline__ int problem_of(const EvArgs &A, unsigned long long gi)
{
    int lo = 0, hi = A.n_prob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.prefix[mid] <= gi) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The persistent event loop.  MinB sets the register budget (MinB CTAs of
// 256 threads resident per SM); kBatch runs many problems at once, each
// particle resolving its own tables.
template <int MinB, bool kBatch>
__global__ void __launch_bounds__(256, MinB) k_event(const EvTables V0, const EvArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int P = A.tile;
    const int H = P;
    Tile T;
    T.base = smem;
    T.P = P;
    T.nsum = A.smem_sums ? V0.n_bins : 0;
    __shared__ int s_nlive, s_novf, s_nhfree, s_status, s_nqc, s_nqx, s_rank;
    __shared__ int s_take_ovf, s_got, s_ovf_base, s_hfree_base, s_exhausted;
    __shared__ unsigned long long s_hist_base;

    Ctx C;
    C.V = &V0;
    C.A = &A;
    C.T = T;
    C.s_status = &s_status;
    C.s_novf = &s_novf;
    C.s_nlive = &s_nlive;
    C.s_nhfree = &s_nhfree;
    C.reg_mask = false;
    C.tmask = 0ull;
    C.tmask1 = 0ull;
    C.cbin = -1;
    C.cval = 0.0;
    __shared__ uint32_t s_cnt[cnt_words(256)];
    C.cnt.base = cnt_column(s_cnt, threadIdx.x);
    for (int i = 0; i < kNumCounters; ++i) C.cnt[i] = 0;
    auto tab = [&](int prob) -> const EvTables & { return kBatch ? A.tabs[prob] : V0; };
    auto seed_of = [&](int prob) -> uint64_t { return kBatch ? A.seeds[prob] : A.seed; };

    for (int s = threadIdx.x; s < P; s += blockDim.x) {
        T.hs()[s] = -1;
        T.hfree()[s] = s;
        T.live()[s] = 0;
    }
    if (A.smem_sums)
        for (int b = threadIdx.x; b < 2 * V0.n_bins; b += blockDim.x) T.ssum()[b] = 0.0;
    if (threadIdx.x == 0) {
        s_nlive = 0; s_novf = 0; s_nhfree = H; s_status = 0; s_nqc = 0; s_nqx = 0;
        s_exhausted = 0;
    }
    __syncthreads();
    OvfP *ovf = A.ovf + (size_t)blockIdx.x * A.ovf_cap;

    for (;;) {
        // ---------------- refill ----------------
        // one thread books the refill; every read of the previous event's
        // queue counters happened before the barrier that closed it
        if (threadIdx.x == 0) {
            s_nqc = 0;
            s_nqx = 0;
            if (s_novf > A.ovf_cap) s_novf = A.ovf_cap;
            const int free_slots = P - s_nlive;
            const int take = min(free_slots, s_novf);
            s_take_ovf = take;
            s_ovf_base = s_novf - take;
            s_novf -= take;
            const int need = free_slots - take;
            int got = 0;
            if (need > 0 && s_novf == 0 && !s_exhausted && s_status == 0) {
                const unsigned long long g0 = atomicAdd(A.next, (unsigned long long)need);
                if (g0 >= A.n) {
                    s_exhausted = 1;
                } else {
                    got = (int)min((unsigned long long)need, A.n - g0);
                    if (g0 + (unsigned long long)need >= A.n) s_exhausted = 1;
                }
                s_hist_base = g0;
            }
            s_got = got;
            s_nhfree -= got;
            s_hfree_base = s_nhfree;
            s_nlive += take + got;
            s_rank = 0;
        }
        __syncthreads();
        {
            // one event adds at most 2^16 + a few to a counter: hand the
            // 32-bit counters to the global 64-bit ones well before they wrap
            uint32_t big = 0;
            for (int i = 0; i < kNumCounters; ++i) big |= C.cnt[i];
            if (big >= (1u << 30))
                for (int i = 0; i < kNumCounters; ++i) {
                    atomicAdd(A.counters + i, (unsigned long long)C.cnt[i]);
                    C.cnt[i] = 0;
                }
        }
        if (s_nlive == 0 && s_novf == 0 && (s_exhausted || s_status != 0)) break;
        if (s_status != 0) break;
        // ---------------- refill + advance ----------------
        // the thread that refills slot s also advances it, so no barrier
        // separates the two
        for (int s0 = 0; s0 < P; s0 += blockDim.x) {
            const int s = s0 + threadIdx.x;
            const bool is_free = s < P && T.hs()[s] < 0;
            const int r = warp_append(&s_rank, is_free);
            if (is_free) {
                PState p;
                if (r < s_take_ovf) {
                    const OvfP &o = ovf[s_ovf_base + r];
                    p.x = o.x; p.y = o.y; p.z = o.z; p.u = o.u; p.v = o.v; p.w = o.w;
                    p.E = o.E; p.wt = o.wt; p.t = o.t; p.cell = o.cell; p.surf = o.surf;
                    p.hslot = o.hslot; p.g = o.g; p.id = o.id; p.ev = 0u;
                    p.prob = T.hprob()[o.hslot];
                    store_p(T, s, p);
                    C.cnt[C_PART]++;
                } else if (r - s_take_ovf < s_got) {
                    const int k = r - s_take_ovf;
                    const int hslot = T.hfree()[s_hfree_base + k];
                    const unsigned long long gi = s_hist_base + (unsigned long long)k;
                    int prob = 0;
                    uint64_t hist = A.first + gi;
                    if (kBatch) {
                        prob = problem_of(A, gi);
                        hist = gi - A.prefix[prob];
                    }
                    T.hidx()[hslot] = hist;
                    T.hprob()[hslot] = prob;
                    T.live()[hslot] = 1;
                    sample_source(tab(prob), seed_of(prob), hist, p);
                    p.hslot = hslot;
                    p.prob = prob;
                    store_p(T, s, p);
                    C.cnt[C_PART]++;
                }
            }
            const bool live = s < P && T.hs()[s] >= 0;
            int kind = 0;   // 1 collide, 2 cross
            if (live) {
                PState p;
                load_p(T, s, p);
                const EvTables &V = tab(p.prob);
                C.V = &V;
                p.ev += 1u;
                if (p.ev > A.max_events) {        // bounded walk: report, never spin
                    atomicCAS(&s_status, 0, DS_TIMEOUT);
                    p.ev = A.max_events;
                }
                Rng32 R;
                R.init(seed_of(p.prob), T.hidx()[p.hslot], p.id, p.ev, 0u);
                Flight f;
                kind = event_advance<FL_ALL>(C, V, R, p, f);
                if (kind != 0) {
                    T.xi()[s] = f.xa.i;
                    T.frac()[s] = f.xa.f;
                    T.ss()[s] = f.ss;
                    T.sc()[s] = f.sc;
                    if (R.cached) {   // the collision continues this Philox block
                        T.b0()[s] = R.blk.x; T.b1()[s] = R.blk.y; T.b2()[s] = R.blk.z; T.b3()[s] = R.blk.w;
                    }
                    T.gi()[s] = f.S;
                    T.sense()[s] = f.sense;
                    T.sig()[s] = f.sig;
                }
                store_p(T, s, p);
            }
            const int pc = warp_append(&s_nqc, kind == 1);
            if (kind == 1) T.qc()[pc] = (unsigned short)s;
            const int px = warp_append(&s_nqx, kind == 2);
            if (kind == 2) T.qx()[px] = (unsigned short)s;
        }
        __syncthreads();

        // ---------------- collide ----------------
        // the warp's lanes step through the queue together, so that the
        // free-gas target sampling can share the work across the warp
        const int nqc = s_nqc;
        for (int j0 = 0; j0 < nqc; j0 += blockDim.x) {
            const int j = j0 + threadIdx.x;
            const bool act = j < nqc;
            const int s = act ? T.qc()[j] : 0;
            PState p;
            Rng32 R;
            R.init(0u, 0u, 0u, 0u, 0u);
            FgState g;
            int cst = 0;
            if (act) {
                load_p(T, s, p);
                const EvTables &V = tab(p.prob);
                C.V = &V;
                R.init(seed_of(p.prob), T.hidx()[p.hslot], p.id, p.ev, 1u);
                const int m = V.cell_mat[p.cell];
                if (m >= 0) R.preload(T.b0()[s], T.b1()[s], T.b2()[s], T.b3()[s]);
                Flight f;
                f.sig = T.sig()[s];
                f.ss = T.ss()[s];
                f.sc = T.sc()[s];
                f.xa = XsAt{m, T.xi()[s], T.frac()[s]};
                cst = event_collide_begin<FL_ALL>(C, V, R, p, f, g);
            }
            float Vt = 0.f, mu = 0.f;
            if (!warp_free_gas(C, cst == 2, R, g, Vt, mu) && cst == 2) {
                atomicCAS(&s_status, 0, DS_TIMEOUT);
                cst = 1;
            }
            if (act) {
                if (cst != 0 && event_collide_end(C, R, p, cst, g, Vt, mu)) store_p(T, s, p);
                else particle_dies(C, s, p.hslot);
            }
        }

        // ---------------- cross ----------------
        const int nqx = s_nqx;
        for (int j = threadIdx.x; j < nqx; j += blockDim.x) {
            const int s = T.qx()[j];
            PState p;
            load_p(T, s, p);
            const EvTables &V = tab(p.prob);
            C.V = &V;
            Rng32 R;
            R.init(seed_of(p.prob), T.hidx()[p.hslot], p.id, p.ev, 1u);
            Flight f;
            f.S = T.gi()[s];
            f.sense = T.sense()[s];
            // split copies wait in the CTA's overflow bank
            auto push = [&](const PState &q, uint32_t cid) -> bool {
                const int slot = atomicAdd(&s_novf, 1);
                if (slot >= A.ovf_cap) return false;
                OvfP o;
                o.x = q.x; o.y = q.y; o.z = q.z; o.u = q.u; o.v = q.v; o.w = q.w;
                o.E = q.E; o.wt = q.wt; o.t = q.t; o.cell = q.cell; o.surf = q.surf;
                o.hslot = q.hslot; o.g = q.g;
                o.id = cid;
                ovf[slot] = o;
                atomicAdd(&T.live()[q.hslot], 1);
                return true;
            };
            if (event_cross<FL_ALL>(C, V, R, p, f, push)) store_p(T, s, p);
            else particle_dies(C, s, p.hslot);
        }
        __syncthreads();
    }

    // flush per-CTA sums and counters
    __syncthreads();
    if (A.smem_sums) {
        for (int b = threadIdx.x; b < V0.n_bins; b += blockDim.x) {
            const double sv = T.ssum()[b], qv = T.ssq()[b];
            if (sv != 0.0) atomicAdd(A.sum + b, sv);
            if (qv != 0.0) atomicAdd(A.sq + b, qv);
        }
    }
    if (threadIdx.x == 0 && s_status != 0) atomicCAS(A.status, 0, s_status);
    for (int i = 0; i < kNumCounters; ++i) {
        unsigned long long v = C.cnt[i];   // a warp's sum needs 64 bits
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(A.counters + i, v);
    }
}

// population_control.cpp:55-84 on a thread's own stack, after every walk
// (handler.cpp:27), keyed as the FP64 engines' comb: the first tooth is one
// uniform from the stream of the particle that just walked, at event
// kCombEvent; tooth j is filled in place from entry i >= j (a particle passes
// at most one tooth, the reference's `if`); teeth left over hold the bottom
// entry with its own weight (bank_tmp(teeth, Pbank[0])); the combed copies
// are renamed child_id(walker, kCombEvent, j + 1).  The weights are summed in
// FP64.  Returns the new stack height (teeth).  Out of line: it runs once per
// combed walk, and its loops stay out of the event loop's instruction stream.
constexpr uint32_t kCombEvent = 0xFFFFFFFFu;

__device__ __noinline__ int comb_stack(OvfP *stk, int sp, int teeth, uint64_t seed, uint64_t hist,
                                       uint32_t walker)
{
    double W = 0.0;
    for (int i = 0; i < sp; ++i) W += (double)stk[i].wt;
    const double w_avg = W / (double)teeth;
    Rng32 R;
    R.init(seed, hist, walker, kCombEvent, 0u);
    double tooth = (double)R.next() * w_avg;
    const OvfP first = stk[0];
    double sum = 0.0;
    int j = 0;
    for (int i = 0; i < sp; ++i) {
        sum += (double)stk[i].wt;
        if (sum > tooth && j < teeth) {   // j < teeth: rounding cannot add a tooth
            OvfP q = stk[i];
            q.wt = (float)w_avg;
            stk[j++] = q;
            tooth += w_avg;
        }
    }
    for (int k = j; k < teeth; ++k) stk[k] = first;
    for (int k = 0; k < teeth; ++k) stk[k].id = child_id(walker, kCombEvent, (uint32_t)(k + 1));
    return teeth;
}

// The per-thread loop: each thread carries one particle through event after
// event in registers (advance, then collision or crossing, with the same
// event functions and Philox keying as k_event), keeps its history's split
// copies on its own LIFO stack in HBM, and takes the next history from the
// global counter with one atomic per warp.  No block barrier separates
// events, and no particle state goes through shared memory; shared memory
// holds only the CTA's tally sums.  A history's row is the thread's own, so
// it is folded when the thread finishes the history.

template <int MinB, bool kBatch, int kFl>
__global__ void __launch_bounds__(kTrackBlock, MinB) k_track(const EvTables V0, const EvArgs A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_status;
    Ctx C;
    C.V = &V0;
    C.A = &A;
    C.T.base = smem;   // P = 0: only the sums
    C.T.P = 0;
    C.T.nsum = A.smem_sums ? V0.n_bins : 0;
    C.s_status = &s_status;
    C.s_novf = nullptr;
    C.s_nlive = nullptr;
    C.s_nhfree = nullptr;
    C.reg_mask = A.row_nb <= 128;
    C.tmask = 0ull;
    C.tmask1 = 0ull;
    C.cbin = -1;
    C.cval = 0.0;
    __shared__ uint32_t s_cnt[cnt_words(kTrackBlock)];
    C.cnt.base = cnt_column(s_cnt, threadIdx.x);
    for (int i = 0; i < kNumCounters; ++i) C.cnt[i] = 0;
    auto tab = [&](int prob) -> const EvTables & { return kBatch ? A.tabs[prob] : V0; };
    auto seed_of = [&](int prob) -> uint64_t { return kBatch ? A.seeds[prob] : A.seed; };
    if (A.smem_sums) {
        for (int b = threadIdx.x; b < 2 * V0.n_bins; b += blockDim.x) C.T.ssum()[b] = 0.0;
        if constexpr (kFl == FL_MG) C.T.lane_bin()[threadIdx.x] = -1;
    }
    if (threadIdx.x == 0) s_status = 0;
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int hslot = threadIdx.x;
    const int depth = A.ovf_cap / kTrackBlock;
    OvfP *stk = A.ovf + (size_t)blockIdx.x * A.ovf_cap + (size_t)threadIdx.x * depth;
    int sp = 0;
    bool have = false, open = false, exhausted = false;
    PState p;
    uint64_t hist = 0;
    int prob = 0;
    uint32_t walks = 0;   // particles of the current history (bounded)
    // batches: the bounds of the problem of the lane's last history
    unsigned long long prob_lo = 1, prob_hi = 0;
    // split copies wait on the thread's own stack
    auto push = [&](const PState &q, uint32_t cid) -> bool {
        if (sp >= depth) return false;
        OvfP o;
        o.x = q.x; o.y = q.y; o.z = q.z; o.u = q.u; o.v = q.v; o.w = q.w;
        o.E = q.E; o.wt = q.wt; o.t = q.t; o.cell = q.cell; o.surf = q.surf;
        o.hslot = q.hslot; o.g = q.g;
        o.id = cid;
        stk[sp++] = o;
        return true;
    };
    for (uint32_t it = 1;; ++it) {
        if constexpr (kFl == FL_ALL) {
            // a walk has just ended whenever the stack is non-empty here
            if (!have && sp > 0) {
                const EvTables &Vc = tab(prob);
                if (Vc.comb_teeth > 0 && sp >= Vc.comb_bank_max)
                    sp = comb_stack(stk, sp, Vc.comb_teeth, seed_of(prob), hist, p.id);
            }
        }
        // the next particle: the history's own split copies first (LIFO, as
        // the reference's bank), then a new history
        if (!have && sp > 0) {
            const OvfP o = stk[--sp];
            p.x = o.x; p.y = o.y; p.z = o.z; p.u = o.u; p.v = o.v; p.w = o.w;
            p.E = o.E; p.wt = o.wt; p.t = o.t; p.cell = o.cell; p.surf = o.surf;
            p.hslot = hslot; p.g = o.g; p.id = o.id; p.ev = 0u; p.prob = prob;
            have = true;
            C.cnt[C_PART]++;
            if (++walks > (1u << 24)) atomicCAS(&s_status, 0, DS_TIMEOUT);
        }
        // new histories start together: a lane whose history ended waits
        // until refill_min lanes of its warp are idle (or no lane has work
        // left), so the fold and the source sampling run for many lanes at
        // once instead of for one or two while the rest wait
        const bool idle = !have && !exhausted;
        const unsigned im = __ballot_sync(0xffffffffu, idle);
        const bool refill = __popc(im) >= A.refill_min || __ballot_sync(0xffffffffu, have) == 0u;
        if (refill && !have && open) {
            history_fold<kFl, !kBatch>(C, hslot, prob);
            open = false;
        }
        const bool need = refill && idle;
        // the warp's lanes that need a history take consecutive ones, one
        // each, with one atomic.  In a batch the history index runs over the
        // concatenated problems: a lane looks its problem up when the index
        // leaves the bounds of the last one.  (Taking several consecutive
        // histories per lane, to look problems up less often, measured
        // slower: 8 at a time ran a batch of 4096 uneven shields in 498 ms
        // against 378 ms.)
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(A.next, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const unsigned long long gi = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
                if (gi >= A.n) {
                    exhausted = true;
                } else {
                    if constexpr (kBatch) {
                        if (!(gi >= prob_lo && gi < prob_hi)) {
                            prob = problem_of(A, gi);
                            prob_lo = A.prefix[prob];
                            prob_hi = A.prefix[prob + 1];
                        }
                        hist = gi - prob_lo;
                    } else {
                        prob = 0;
                        hist = A.first + gi;
                    }
                    sample_source(tab(prob), seed_of(prob), hist, p);
                    p.hslot = hslot;
                    p.prob = prob;
                    have = true;
                    open = true;
                    walks = 1;
                    C.cnt[C_PART]++;
                }
            }
        }
        // the warp leaves together: when no lane has work, or on an error
        const bool err = *(volatile int *)&s_status != 0;
        if (__all_sync(0xffffffffu, !have) || __any_sync(0xffffffffu, err)) break;
        Rng32 R;
        R.init(0u, 0u, 0u, 0u, 0u);
        Flight f;
        FgState g;
        int kind = 0, cst = 0;
        if (have) {
            const EvTables &V = tab(prob);
            C.V = &V;
            p.ev += 1u;
            if (p.ev > A.max_events) {        // bounded walk: report, never spin
                atomicCAS(&s_status, 0, DS_TIMEOUT);
                p.ev = A.max_events;
            }
            R.init(seed_of(prob), hist, p.id, p.ev, 0u);
            kind = event_advance<kFl>(C, V, R, p, f);
            if (kind == 1) cst = event_collide_begin<kFl>(C, V, R, p, f, g);
        }
        // free-gas target velocities for the whole warp (every lane takes part)
        float Vt = 0.f, mu = 0.f;
        if constexpr (kFl != FL_MG) {   // multigroup scatters sample no target
            if (!warp_free_gas(C, cst == 2, R, g, Vt, mu) && cst == 2) {
                atomicCAS(&s_status, 0, DS_TIMEOUT);
                cst = 1;
            }
        }
        if (kind == 1) {
            have = cst != 0 && event_collide_end(C, R, p, cst, g, Vt, mu);
        } else if (kind == 2) {
            const EvTables &V = tab(prob);
            C.V = &V;
            R.draw = 1;   // the crossing draws from word 1 on, as in k_event
            have = event_cross<kFl>(C, V, R, p, f, push);
        }
        if ((it & 4095u) == 0) {
            // one event adds at most 2^16 + a few to a counter: hand the
            // 32-bit counters to the global 64-bit ones well before they wrap
            uint32_t big = 0;
            for (int i = 0; i < kNumCounters; ++i) big |= C.cnt[i];
            if (big >= (1u << 30))
                for (int i = 0; i < kNumCounters; ++i) {
                    atomicAdd(A.counters + i, (unsigned long long)C.cnt[i]);
                    C.cnt[i] = 0;
                }
        }
    }

    if constexpr (kFl == FL_MG) {
        if (A.smem_sums) {   // the thread's running sums into the CTA's
            const int lb = C.T.lane_bin()[threadIdx.x];
            if (lb >= 0) {
                atomicAdd(C.T.ssum() + lb, C.T.lane_acc()[2 * threadIdx.x]);
                atomicAdd(C.T.ssq() + lb, C.T.lane_acc()[2 * threadIdx.x + 1]);
            }
        }
    }
    __syncthreads();
    if (A.smem_sums) {
        for (int b = threadIdx.x; b < V0.n_bins; b += blockDim.x) {
            const double sv = C.T.ssum()[b], qv = C.T.ssq()[b];
            if (sv != 0.0) atomicAdd(A.sum + b, sv);
            if (qv != 0.0) atomicAdd(A.sq + b, qv);
        }
    }
    if (threadIdx.x == 0 && s_status != 0) atomicCAS(A.status, 0, s_status);
    for (int i = 0; i < kNumCounters; ++i) {
        unsigned long long v = C.cnt[i];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && v) atomicAdd(A.counters + i, v);
    }
}

template <int kFl>
EvKernel pick_track(int minb, bool batch)
{
    if (batch)
        return minb == 4 ? k_track<4, true, kFl>
             : minb == 6 ? k_track<6, true, kFl> : minb == 7 ? k_track<7, true, kFl> : k_track<8, true, kFl>;
    return minb == 4 ? k_track<4, false, kFl>
         : minb == 6 ? k_track<6, false, kFl> : minb == 7 ? k_track<7, false, kFl> : k_track<8, false, kFl>;
}

}  // namespace
}  // namespace mc
