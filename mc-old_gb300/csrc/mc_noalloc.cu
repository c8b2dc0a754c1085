// mc_noalloc.cu -- FP64 replay that allocates no device memory.
//
// mc_run() grows its scratch (per-history tally rows, split-particle stacks,
// counters) with cudaMalloc on first use.  Some callers cannot allow that
// once they are running: a host whose device memory belongs to another
// allocator (a framework's caching pool with a fixed budget), or a service
// that reserves everything at start-up and forbids allocation on its request
// path.  mc_run_replay_noalloc() gives them the FP64 replay transport with
// its scratch in one file-scope device array of fixed size instead.  The
// problem tables are the handle's (allocated when the problem was loaded);
// the tally sums go to buffers the caller passes.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "mc_device.h"
#include "mc_engine.h"
#include "mc_handle.h"
#include "mcgpu.h"

namespace mc {

namespace {

constexpr size_t kScratchBytes = 64ull << 20;     // MC_NOALLOC_SCRATCH_BYTES
constexpr size_t kCtrlBytes = 4096;
// 96 blocks of 128: fewer CTAs than the GPU has SMs, because the split
// stacks of every thread must fit the fixed array; this path trades
// throughput against mc_run's replay for allocating nothing
constexpr int kThreads = 12288;
constexpr int kBlock = 128;
constexpr uint32_t kDepth = 16;                  // split copies per history
constexpr uint32_t kMinChunk = 1024;             // histories per fold, at least

// The scratch: control words, split stacks, per-history tally rows.  Every
// GPU that loads the library holds these 64 MiB until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (host code cannot use the symbol's name as an address).
cudaError_t scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace

}  // namespace mc

using namespace mc;

extern "C" mc_status mc_run_replay_noalloc(mc_problem *p, uint64_t first, uint64_t n, uint64_t seed,
                                           double *d_sum, double *d_sumsq)
{
    if (!p || !d_sum || !d_sumsq) return MC_ERR_ARG;
    if (!p->dev.ready) { p->err = "problem was not loaded"; return MC_ERR_ARG; }
    DeviceProblem &d = p->dev;
    if (d.dt.comb_teeth > (int)kDepth / 2) {
        p->err = "mc_run_replay_noalloc: a particle comb with more than " + std::to_string(kDepth / 2) +
                 " teeth does not fit the fixed split stack";
        return MC_ERR_ARG;
    }
    const long long nb = std::max<long long>(d.dt.n_bins, 1);
    const size_t stack_bytes = (size_t)kThreads * kDepth * fp64_particle_bytes();
    const size_t row_bytes = (size_t)nb * sizeof(double);
    if (kCtrlBytes + stack_bytes + (size_t)kMinChunk * row_bytes > kScratchBytes) {
        p->err = "mc_run_replay_noalloc: " + std::to_string(nb) + " tally bins need more than the " +
                 std::to_string(kScratchBytes >> 20) + " MiB static scratch holds (at most " +
                 std::to_string((kScratchBytes - kCtrlBytes - stack_bytes) / ((size_t)kMinChunk * sizeof(double))) +
                 " bins)";
        return MC_ERR_ARG;
    }
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) { p->err = cuda_msg(e, "cudaGetSymbolAddress(noalloc scratch)"); return MC_ERR_CUDA; }
    char *b = static_cast<char *>(base);
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(b);
    int *status = reinterpret_cast<int *>(b + 128);
    unsigned int *next = reinterpret_cast<unsigned int *>(b + 192);
    void *stack = b + kCtrlBytes;
    double *hist = reinterpret_cast<double *>(b + kCtrlBytes + stack_bytes);
    const uint64_t chunk = (kScratchBytes - kCtrlBytes - stack_bytes) / row_bytes;

    // the array keeps the previous call's contents: clear what starts at zero
    // (the caller's arrays hold exactly n_bins doubles, none when n_bins is 0)
    const size_t out_bytes = (size_t)d.dt.n_bins * sizeof(double);
    if ((e = cudaMemsetAsync(b, 0, kCtrlBytes, d.stream)) != cudaSuccess ||
        (out_bytes && (e = cudaMemsetAsync(d_sum, 0, out_bytes, d.stream)) != cudaSuccess) ||
        (out_bytes && (e = cudaMemsetAsync(d_sumsq, 0, out_bytes, d.stream)) != cudaSuccess)) {
        p->err = cuda_msg(e, "mc_run_replay_noalloc memset");
        return MC_ERR_CUDA;
    }
    for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
        const uint32_t cn = (uint32_t)std::min<uint64_t>(chunk, n - c0);
        HistoryArgs A;
        A.first = first + c0;
        A.n = cn;
        A.seed = seed;
        A.hist = hist;
        A.stack = stack;
        A.stack_depth = kDepth;
        A.counters = cnt;
        A.digest = nullptr;
        A.status = status;
        A.next = next;
        if ((e = cudaMemsetAsync(next, 0, sizeof(unsigned int), d.stream)) != cudaSuccess ||
            (e = launch_history_fp64(d.dt, A, true, kThreads / kBlock, kBlock, d.stream)) != cudaSuccess ||
            (e = launch_fold(hist, cn, d.dt.n_bins, d_sum, d_sumsq, true, d.stream)) != cudaSuccess) {
            p->err = cuda_msg(e, "mc_run_replay_noalloc launch");
            return MC_ERR_CUDA;
        }
    }
    int hs = 0;
    unsigned long long c[kNumCounters];
    if ((e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(c, cnt, sizeof(c), cudaMemcpyDeviceToHost, d.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(d.stream)) != cudaSuccess) {
        p->err = cuda_msg(e, "mc_run_replay_noalloc");
        return MC_ERR_CUDA;
    }
    if (hs != DS_OK) {
        p->err = hs == DS_OVERFLOW
                     ? "mc_run_replay_noalloc: more than " + std::to_string(kDepth) +
                           " particles pending on one history's stack (comb teeth plus split copies)"
                     : std::string("mc_run_replay_noalloc: ") + device_status_text(hs);
        return status_from_device(hs);
    }
    mc_counters &L = d.last;
    std::memset(&L, 0, sizeof(L));
    L.flights = c[0]; L.collisions = c[1]; L.crossings = c[2]; L.tally_updates = c[3];
    L.particles = c[4]; L.splits = c[5]; L.xs_evals = c[6]; L.freegas_iters = c[7];
    L.nuc_lookups = c[8];
    L.histories = n;
    return MC_OK;
}
