// mc_engine.h -- host-side run orchestration: device tables, accumulated
// tallies, scratch buffers and the per-mode drivers.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "mcgpu.h"
#include "mc_device.h"
#include "mc_problem.h"

namespace mc {

// A device buffer that only grows.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct EventState;   // mixed-precision event engine (mc_event.cu)
struct BankState;    // its event-split engine over an HBM particle bank (mc_bank.cu)
struct EvTables;     // the mixed-precision engine's FP32 tables (mc_evtables.h)
struct BatchState;   // batches of problems in one persistent launch (mc_event.cu)

struct DeviceProblem {
    bool ready = false;
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    void *blob = nullptr;          // every problem table, one allocation
    void *h_blob = nullptr;        // pinned host copy of blob
    size_t blob_bytes = 0;
    DevTables dt{};
    double *d_sum = nullptr;       // [n_bins] sum of history totals
    double *d_sq = nullptr;        // [n_bins] sum of squared history totals
    long long *d_exact = nullptr;  // [n_bins][2][kExactLimbs] exact sums of the FP64 runs
    bool exact_valid = true;       // every run since the last reset added to d_exact
    uint64_t histories = 0;        // histories folded into d_sum / d_sq
    uint64_t ntrack = 0;           // flights over all runs (the reference's Ntrack)
    mc_counters last{};
    std::vector<uint64_t> digests; // last FP64 run with record_digests
    // FP64 history-engine scratch
    DevBuf hist, stack, digest, misc;
    // event engine (owned)
    EventState *ev_state = nullptr;
    BankState *bank_state = nullptr;   // event-split engine buffers (owned)
    mc_tune tuned{};               // launch shape picked by mc_autotune (0 = defaults)
    void *lr = nullptr;            // forward / backward scratch (mc_lr.cpp)
};

mc_status device_problem_init(const Tables &t, DeviceProblem &d, std::string &err);
void device_problem_free(DeviceProblem &d);
mc_status reset_tallies(DeviceProblem &d, std::string &err);
mc_status upload_tables(DeviceProblem &d, std::string &err);
// the same on a caller's stream, without waiting (batches queue many problems)
cudaError_t upload_tables_async(DeviceProblem &d, cudaStream_t st);
cudaError_t reset_tallies_async(DeviceProblem &d, cudaStream_t st);
cudaError_t event_tables_upload_async(DeviceProblem &d, cudaStream_t st);
mc_status read_sums(const DeviceProblem &d, std::vector<double> &sum, std::vector<double> &sq, std::string &err);
mc_status run_histories(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed,
                        mc_mode mode, const mc_tune *tune, std::string &err);

// grows buf to at least bytes (contents are not kept)
bool devbuf_reserve(DevBuf &buf, size_t bytes);
void devbuf_free(DevBuf &buf);

// FP64 history engine (mc_engine.cpp)
mc_status run_fp64(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed, bool replay,
                   const mc_tune *tune, std::string &err);
// mixed-precision event engine (mc_event.cu)
mc_status run_event(const Tables &t, DeviceProblem &d, uint64_t first, uint64_t n, uint64_t seed,
                    const mc_tune *tune, std::string &err);
void event_state_free(EventState *s);
// the event-split engine (mc_tune.kernel = 3) on one problem's FP32 tables
// may_split: cells differ in importance, so a history can own several particles
mc_status run_bank(DeviceProblem &d, const EvTables &V, int flavor, bool may_split, uint64_t first, uint64_t n,
                   uint64_t seed, const mc_tune *tune, std::string &err);
void bank_state_free(BankState *b);
bool event_tables_ready(const Tables &t, DeviceProblem &d, std::string &err);
// copies the mixed-precision engine's tables again from pinned host memory
// (nothing before that engine first ran) and their size in bytes
mc_status event_tables_upload(DeviceProblem &d, std::string &err);
size_t event_table_bytes(const DeviceProblem &d);

// batches (mc_event.cu)
// sums_to (nullable): 2 device arrays per problem (sum, sumsq) to fold into
// instead of the problems' own tallies (used while autotuning)
mc_status batch_create(const std::vector<const Tables *> &tabs, const std::vector<DeviceProblem *> &probs,
                       const uint64_t *hist, const std::vector<double *> *sums_to, BatchState **out,
                       std::string &err);
cudaStream_t batch_stream(const BatchState *b);
mc_status batch_run(BatchState *b, int device_sms, uint64_t seed, const mc_tune *tune, const mc_tune &tuned,
                    std::string &err);
void batch_state_free(BatchState *b);
const mc_counters &batch_counters(const BatchState *b);
uint64_t batch_problem_seed(uint64_t seed, uint32_t i);

mc_status status_from_device(int ds);
// message for a device status word (DS_*) of the FP64 history kernels
const char *device_status_text(int ds);
// nearest double (ties to even) of one exact value of kExactLimbs limbs (mc_exact.cu)
double exact_round(const int64_t *limbs);
void lr_scratch_free(void *lr);
std::string cuda_msg(cudaError_t e, const char *what);

}  // namespace mc
