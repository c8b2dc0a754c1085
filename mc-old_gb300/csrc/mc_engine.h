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
    uint64_t histories = 0;        // histories folded into d_sum / d_sq
    uint64_t ntrack = 0;           // flights over all runs (the reference's Ntrack)
    mc_counters last{};
    std::vector<uint64_t> digests; // last FP64 run with record_digests
    // FP64 history-engine scratch
    DevBuf hist, stack, digest, misc;
    // event engine (owned)
    EventState *ev_state = nullptr;
};

mc_status device_problem_init(const Tables &t, DeviceProblem &d, std::string &err);
void device_problem_free(DeviceProblem &d);
mc_status reset_tallies(DeviceProblem &d, std::string &err);
mc_status upload_tables(DeviceProblem &d, std::string &err);
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

mc_status status_from_device(int ds);
std::string cuda_msg(cudaError_t e, const char *what);

}  // namespace mc
