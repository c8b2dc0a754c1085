/*
 * mcgpu.h -- C ABI of the GB300 fixed-source particle-history library.
 *
 * Drop-in for the fixed-source path of MC-old's Simulator (C++, in-process):
 * each entry point names the reference interface it replaces.  Plain C types
 * only: no C++ or framework types cross this boundary.
 *
 * Conventions
 *  - Every call returns an mc_status; nothing exits or throws across the ABI
 *    (the reference calls std::exit or a bare throw, setup.cpp:235,579;
 *    general.cpp:33).  mc_last_error() gives the message of the last failure
 *    on a handle.
 *  - The library owns device memory; the caller owns every output buffer.
 *  - One mc_problem per host thread.  Calls on one handle are not re-entrant.
 *    Each handle has its own CUDA stream.
 *  - Results are deterministic for a given (seed, history range, mode).
 *  - Histories are keyed into a counter-based Philox4x32-10 stream by
 *    (seed, history, particle, event, draw), so any history range can be run
 *    separately and merged ("resume" = run [a, b) then [b, c)).
 */
#ifndef MCGPU_H
#define MCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mc_problem mc_problem;

typedef enum {
    MC_OK = 0,
    MC_ERR_INPUT = 1,     /* malformed or unsupported input.xml / tables */
    MC_ERR_CUDA = 2,      /* CUDA runtime error (no device, launch failure) */
    MC_ERR_OVERFLOW = 3,  /* particle bank or split stack capacity exceeded */
    MC_ERR_LOST = 4,      /* a particle left every cell (general.cpp:31-33) */
    MC_ERR_TIMEOUT = 5,   /* a bounded device-side wait ran out */
    MC_ERR_NAN = 6,       /* non-finite particle weight or position */
    MC_ERR_NOMEM = 7,     /* host or device allocation failed */
    MC_ERR_ARG = 8        /* bad argument (null pointer, index out of range) */
} mc_status;

typedef enum {
    /* FP64 history-based, the reference's arithmetic order, portable
     * elementary functions, tallies folded in history order: every history's
     * event sequence and every tally bin equal the CPU oracle's bit for bit. */
    MC_FP64_REPLAY = 0,
    /* FP64 history-based with the GPU's native FP64 libm and a tree fold:
     * the plain double-precision GPU history path. */
    MC_FP64_PLAIN = 1,
    /* FP32 tracking, FP64 tally accumulation.  Three engines: a persistent
     * tile of particles per CTA (structure of arrays in shared memory,
     * ballot/prefix-sum compacted collision and crossing queues); one
     * particle per thread in registers; or the particle bank as a structure
     * of arrays in HBM with one kernel per event type (advance, collide,
     * cross) over queues compacted with warp ballots and prefix sums.  All
     * sample free-gas targets for a whole warp at once and follow the same
     * tracks.  mc_tune.kernel or mc_autotune picks one; the default is the
     * per-thread kernel.  A problem with the particle comb
     * (population_control.cpp:55-84) runs on the per-thread kernel, which
     * keeps each history's bank on its thread's stack. */
    MC_MIXED_EVENT = 2
} mc_mode;

/* Launch / capacity knobs.  Pass NULL to mc_run for the defaults (or the
 * values picked by mc_autotune). */
typedef struct {
    uint32_t block;          /* threads per block (0 = default) */
    uint32_t grid_blocks;    /* blocks, 0 = fill the GPU */
    uint32_t stack_depth;    /* split-particle stack per thread: FP64 modes and the
                                per-thread event kernel (0 = 32, or teeth + 32
                                with the particle comb); the tile kernel: split
                                copies its CTA's overflow bank holds (0 = 4 per
                                tile particle); the event-split engine: split
                                copies its stack holds (0 = a quarter of the
                                bank's slots, at least 4096) */
    uint32_t chunk;          /* FP64 modes: histories per fold chunk (0 = auto) */
    uint32_t bank_capacity;  /* event mode: particles per CTA tile (0 = tuned / 512);
                                the event-split engine: particle slots of the
                                HBM bank, a multiple of 256 in 1024..2^24
                                (0 = 2^20) */
    uint32_t record_digests; /* FP64 modes: keep per-history event digests */
    uint32_t blocks_per_sm;  /* event mode: resident CTAs per SM, which sets the
                                register budget: 2, 3 or 4 for the tile kernel
                                (256 threads), 4, 6, 7 or 8 for the per-thread
                                kernel (128 threads); 0 = tuned / 4 / 8 */
    uint32_t kernel;         /* event mode: 1 = particle tile with event queues,
                                2 = one particle per thread, 3 = event kernels
                                over an HBM particle bank, 0 = tuned / 2; the
                                tile kernel and the event-split engine refuse
                                the particle comb, and batches run kernel 1
                                or 2 */
    uint32_t max_events;     /* events one particle may take before the run stops
                                with MC_ERR_TIMEOUT (0 = 2^22); a small cap
                                exercises that path on purpose */
    uint32_t refill;         /* per-thread event kernel: a lane that finished its
                                history waits until this many lanes of its warp
                                are idle, so that they fold and start histories
                                together (1..32; 0 = 8 for multigroup problems,
                                4 otherwise) */
} mc_tune;

/* Event counters and timing of the last mc_run.  The counts follow the
 * reference's own bookkeeping: flights is its Ntrack (simulator.h:109,
 * general.cpp:76). */
typedef struct {
    uint64_t flights;         /* move_particle calls */
    uint64_t collisions;
    uint64_t crossings;
    uint64_t tally_updates;   /* per-history bin accumulations */
    uint64_t particles;       /* particles walked, split copies included */
    uint64_t splits;          /* copies made by importance splitting */
    uint64_t xs_evals;        /* macroscopic cross-section evaluations */
    uint64_t freegas_iters;   /* free-gas rejection-loop iterations */
    uint64_t nuc_lookups;     /* sum over flights of the material's nuclide count */
    uint64_t histories;       /* histories in the last run */
    double   transport_ms;    /* device time of the transport kernels */
    double   fold_ms;         /* device time of the history fold */
    double   total_ms;        /* device time of the whole mc_run */
    uint32_t launches;        /* kernels launched by the last mc_run (mixed
                                 mode: 2 where a second kernel adds the
                                 replicated sums of a problem of more than
                                 4096 bins, or of a batch) */
    uint32_t reserved;        /* 0 (pads the struct to 8 bytes) */
} mc_counters;

/* Replaces Simulator::Simulator(io_dir) (src/simulator/setup.cpp:30): reads
 * <io_dir>/input.xml; ZAID tables come from <xs_dir>/<ZAID>.txt, where
 * xs_dir NULL means "./xs_library" as in the reference (setup.cpp:326). */
mc_status mc_problem_load_xml(const char *io_dir, const char *xs_dir, mc_problem **out);

/* Copies every device table of the problem again from the handle's pinned
 * host copies: the FP64 tables and, once the mixed-precision engine has run
 * on the handle, its FP32 tables (to time a cold start, or after the host
 * copy changed).  The reference keeps its tables in host memory only; this
 * has no counterpart there beyond the table construction in
 * Simulator::Simulator. */
mc_status mc_problem_upload(mc_problem *p);

/* Bytes of the device tables of the problem (what mc_problem_upload moves
 * host -> device). */
mc_status mc_problem_table_bytes(const mc_problem *p, uint64_t *bytes);

/* Releases a handle (the reference's Simulator destructor). */
mc_status mc_problem_free(mc_problem *p);

/* Replaces Simulator::start() (src/simulator/handler.cpp:11-48) for the
 * histories [first_history, first_history + n_histories).  Tally sums
 * accumulate across calls; call mc_reset_tallies to start over. */
mc_status mc_run(mc_problem *p, uint64_t first_history, uint64_t n_histories, uint64_t seed,
                 mc_mode mode, const mc_tune *tune);

/* Zeroes the accumulated tally sums and the history count. */
mc_status mc_reset_tallies(mc_problem *p);

/* Checkpoint / resume.  mc_state_save writes the accumulated tallies (per-bin
 * sums of history totals and of their squares), the history count and Ntrack
 * to a flat binary file; mc_state_load puts them into a handle made from the
 * same input (checked by a fingerprint of the problem tables), which then
 * continues with the histories not run yet: running [0, a), saving, loading
 * in another process and running [a, n) gives the tallies of [0, n) (bit for
 * bit in MC_FP64_REPLAY).  No counterpart in the reference, which keeps no
 * state between runs. */
mc_status mc_state_save(const mc_problem *p, const char *path);
mc_status mc_state_load(mc_problem *p, const char *path);

/* ---- exact sums: merging disjoint history ranges bit for bit ------------
 * The reference folds each history into running FP64 sums (sum += h,
 * squared += h * h, Estimator.cpp:339-346); MC_FP64_REPLAY keeps that order,
 * so the sums of two runs over [0, a) and [a, n) differ in the last bits from
 * one run over [0, n) (FP64 addition is not associative).  Alongside, the FP64
 * modes accumulate every bin's sum of history totals and sum of their squares
 * exactly, as integers in units of 2^-1074: each value is MC_EXACT_LIMBS
 * signed 64-bit limbs, value = sum_j limb[j] * 2^(32 j - 1074), normalised
 * (limbs 0..MC_EXACT_LIMBS-2 in [0, 2^32), the last one signed).  Exact sums
 * of disjoint ranges (other handles, processes or GPUs) added limb by limb in
 * any order and rounded once give, bit for bit, the rounded exact sums of one
 * run over the union: this is the single exchange of a multi-GPU run ("merge
 * on exact integer accumulators").  No counterpart in the reference, which
 * runs on one core. */
#define MC_EXACT_LIMBS 68

/* The exact sums of every bin since the last mc_reset_tallies:
 * limbs[(b * 2 + k) * MC_EXACT_LIMBS + j], k = 0 sum of history totals,
 * k = 1 sum of their squares; cap >= n_bins * 2 * MC_EXACT_LIMBS.  Refused
 * (MC_ERR_ARG) after a mixed-mode or batch run or mc_state_load since that
 * reset: those add to the FP64 sums only. */
mc_status mc_exact_sums_read(const mc_problem *p, int64_t *limbs, uint64_t cap);

/* Rounds n_values exact values (MC_EXACT_LIMBS limbs each, normalised or not,
 * e.g. limb-wise sums over ranks) to the nearest double, ties to even.  Host
 * arithmetic only. */
mc_status mc_exact_round(const int64_t *limbs, uint64_t n_values, double *out);

/* Number of estimators (the reference's Estimators.size(), simulator.h:122). */
mc_status mc_tally_count(const mc_problem *p, uint32_t *n_estimators);

/* Bins of estimator est (Estimator::tally_size, Estimator.cpp:429-432). */
mc_status mc_tally_size(const mc_problem *p, uint32_t est, uint64_t *n_bins);

/* Name of estimator est (the XML name attribute, setup.cpp:641-642). */
mc_status mc_estimator_name(const mc_problem *p, uint32_t est, char *buf, size_t cap);

/* Replaces Estimators[est]->tally(j).mean / .uncer (Estimator.cpp:347-367,
 * 424-427): mean and standard error over the histories run so far, plus the
 * raw per-bin sums of history totals and of their squares.  Any output
 * pointer may be NULL; cap is the capacity of each non-NULL array. */
mc_status mc_tally_read(const mc_problem *p, uint32_t est, double *mean, double *sigma,
                        double *sum, double *sumsq, uint64_t cap);

/* Counters of the last run (Ntrack plus the per-event counts). */
mc_status mc_counters_read(const mc_problem *p, mc_counters *out);

/* Per-history event digests of the last FP64 run made with
 * tune->record_digests (n entries, one per history in run order). */
mc_status mc_digests_read(const mc_problem *p, uint64_t *out, uint64_t cap);

/* Histories requested in the input (<description samples>, setup.cpp:50). */
mc_status mc_nsample(const mc_problem *p, uint64_t *nsample);

/* Histories folded into the tallies so far. */
mc_status mc_histories_run(const mc_problem *p, uint64_t *n);

/* Replaces Simulator::report(io_dir) (src/simulator/report.cpp:9-50): writes
 * the output.h5 group/dataset layout (/summary, one group per estimator with
 * its filter grids and <score>/mean, <score>/uncertainty) as a JSON file at
 * path, HDF5 not being available. */
mc_status mc_report(const mc_problem *p, const char *path);

/* FP64 replay of histories [first_history, first_history + n_histories)
 * that allocates no device memory.  No counterpart in the reference: it is
 * for callers that cannot allocate device memory once running (a host whose
 * device memory belongs to another allocator's fixed pool, or a service that
 * reserves everything at start-up).  The problem must already be loaded; the
 * scratch (split stacks and per-history tally rows) lives in one fixed
 * 64 MiB device array inside the library, held by every GPU that loads the
 * library until the process exits.  Writes the per-bin sums of history
 * totals and of their squares over the range to the caller's device arrays
 * d_sum / d_sumsq (n_bins doubles each, all estimators in order, overwritten),
 * equal bit for bit to what mc_run in MC_FP64_REPLAY adds for the same
 * range; the handle's own tallies are not touched.  Problems with more tally
 * bins than the scratch holds are refused with MC_ERR_ARG.  The first call on
 * a device looks up the array's device address once and keeps it for the
 * life of the process; make that call before any stream capture.  The kept
 * address belongs to the device's primary context: after cudaDeviceReset (or
 * after that context is released and created again) it is stale, so do not
 * call this entry point again in that process.  The grid is 96 blocks of 128
 * threads (the split stacks of every thread live in the fixed array), so
 * throughput is below mc_run's replay.  Every call shares the one array, so
 * calls that overlap on the GPU (two host threads, two handles) race;
 * serialise them. */
mc_status mc_run_replay_noalloc(mc_problem *p, uint64_t first_history, uint64_t n_histories,
                                uint64_t seed, double *d_sum, double *d_sumsq);

/* Picks the mixed-precision engine's kernel and launch shape (tile kernel:
 * particles per CTA tile and resident CTAs per SM; per-thread kernel:
 * resident CTAs per SM, then its refill threshold among 2, 4, 8 and 16;
 * the event-split engine is not sampled) for this problem by timing sample_histories in each
 * candidate shape (at least 4 histories per thread of the largest shape, so
 * that no shape is timed half idle; 0 = 8 per thread); the winner becomes
 * the handle's default for
 * MC_MIXED_EVENT runs made with tune == NULL and is copied to *out.  The
 * problem's tallies are left as they were.  No counterpart in the reference
 * (it has no launch parameters). */
mc_status mc_autotune(mc_problem *p, uint64_t sample_histories, uint64_t seed, mc_tune *out);

/* ---- tally derivatives (one-group multigroup problems) -------------------
 * No counterpart in the reference.  The parameters are every material's
 * one-group (Sigma_s, Sigma_a) in input order: params[2m], params[2m+1]
 * (1/cm for a material written with <multigroup>).  Both calls run FP64
 * replay histories [0, n) keyed by seed and leave the problem's own tallies
 * untouched; runs at different parameters with the same (n, seed) use common
 * random numbers. */

/* The problem's own parameters (2 per material). */
mc_status mc_lr_params(const mc_problem *p, double *params, uint32_t cap);

/* Every tally bin (all estimators in order) at the given parameters: mean and
 * standard error (either pointer may be NULL). */
mc_status mc_forward(mc_problem *p, const double *params, uint64_t n_histories, uint64_t seed,
                     double *tally_out, double *sigma_out);

/* d(tally bin b)/d(param k) at the given parameters by the likelihood-ratio
 * (differential-operator) kernel, dtally[b * n_params + k], with its
 * standard error in sigma (nullable).  n_params = 2 x materials. */
mc_status mc_backward(mc_problem *p, const double *params, uint64_t n_histories, uint64_t seed,
                      double *dtally, double *sigma);

/* mc_backward plus the density derivatives in the same run:
 * drho[b * n_materials + m] = rho_m d(tally bin b)/d rho_m, the derivative
 * with respect to the material's density relative to its value (a density
 * scales both cross sections of the material, so per history it is
 * Sigma_s,m d/dSigma_s,m + Sigma_a,m d/dSigma_a,m), with its standard error
 * in drho_sigma.  Any of the four output pointers may be NULL (not both
 * dtally and drho). */
mc_status mc_backward_density(mc_problem *p, const double *params, uint64_t n_histories, uint64_t seed,
                              double *dtally, double *sigma, double *drho, double *drho_sigma);

/* ---- batches: many independent problems in one persistent launch ---------
 * No counterpart in the reference, which runs one Simulator at a time.  A
 * batch is a list of loaded problems with a history count each; mc_batch_run
 * runs every history of every problem in ONE launch of the event engine
 * (MC_MIXED_EVENT), replayed from a CUDA graph captured at the first run,
 * and folds each problem's results into that problem's tallies (read them
 * with mc_tally_read on the problem handles).  Histories fold into up to 64
 * copies of the batch's bins (one per group of CTAs, at most 256 MiB); a
 * second kernel in the same graph adds the copies into the problems' sums
 * and clears them, so the graph launches two kernels.  Problem i's
 * histories use the seed  seed + 0x9E3779B97F4A7C15 * (i + 1),  so they are
 * the histories an mc_run of that problem alone with that seed would
 * follow.  The problems
 * must outlive the batch and must not be run on their own while a batch run
 * is in flight. */
typedef struct mc_batch mc_batch;

mc_status mc_batch_create(mc_problem *const *problems, uint32_t n, const uint64_t *histories,
                          mc_batch **out);
mc_status mc_batch_run(mc_batch *b, uint64_t seed, const mc_tune *tune);
/* Counters and device time of the last mc_batch_run (summed over problems). */
mc_status mc_batch_counters(const mc_batch *b, mc_counters *out);
/* Times each candidate launch shape on the batch with every problem's
 * histories scaled by sample_fraction (at least 64 each; 0 or out of
 * (0, 1]: 0.05) and keeps the fastest for runs with tune == NULL; the
 * problems' tallies are untouched.
 * The refill threshold keeps its default: the scaled sample holds a
 * different mix of problem sizes, and a threshold it favours did not carry
 * over to the whole batch. */
mc_status mc_batch_autotune(mc_batch *b, uint64_t seed, double sample_fraction, mc_tune *out);
/* Batch-wide forms of mc_problem_upload, mc_reset_tallies and mc_tally_read,
 * for callers that move every problem's tables and tallies at each run: the
 * copies and clears of all problems are queued on the batch's stream and
 * waited for once, instead of once per problem.  mc_batch_tally_read writes
 * every problem's bins (all its estimators in order), problem after problem,
 * into each non-NULL array of cap >= the batch's total bins, with the
 * statistics of mc_tally_read over each problem's own histories.  Each call
 * first waits for every problem's own stream.  No counterpart in the
 * reference. */
mc_status mc_batch_upload(mc_batch *b);
mc_status mc_batch_reset(mc_batch *b);
mc_status mc_batch_tally_read(mc_batch *b, double *mean, double *sigma, double *sum, double *sumsq, uint64_t cap);
mc_status mc_batch_free(mc_batch *b);
const char *mc_batch_last_error(const mc_batch *b);

/* Human-readable message for the last failing call on p (never NULL). */
const char *mc_last_error(const mc_problem *p);

/* Static name of a status code. */
const char *mc_status_string(mc_status s);

#ifdef __cplusplus
}
#endif
#endif /* MCGPU_H */
