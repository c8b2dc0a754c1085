// mc_device.h -- device view of the problem tables and the kernel entry
// points of the library (host-callable launch wrappers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mc {

// Plain-pointer view of Tables (mc_problem.h) in device memory.  Every array
// lives in one allocation; the layouts are those documented in mc_problem.h.
struct DevTables {
    int n_surf, n_cell, n_mat, n_nuc, mg_groups, n_est, n_src;
    long long n_bins;
    double wr, ws;
    int comb_bank_max, comb_teeth;     // particle comb (0 teeth: off)
    const int *surf_type, *surf_bc;
    const double *surf_coef;
    const double *cell_imp;
    const int *cell_mat, *cell_surf_off, *cell_surf, *cell_sense;
    const int *cell_tl_off, *cell_tl, *cell_c_off, *cell_c, *surf_est_off, *surf_est;
    const int *mat_off, *mat_nuc;
    const double *mat_dens;
    const int *nuc_kind, *nuc_len;
    const double *nuc_A, *nuc_const;
    const long long *nuc_off;
    const double *xs_E, *xs_S, *xs_C, *xs_T;
    const double *mg_total, *mg_scatter, *mg_scat_tot, *mg_capture;
    const int *est_score_off, *score_kind, *score_kernel;
    const int *est_filt_off, *filt_kind, *filt_size, *filt_grid_len;
    const long long *filt_grid_off;
    const double *filt_grid, *est_factor;
    const int *est_factor_off;
    const long long *est_bin_off;
    const double *src_pos, *src_dir_par, *src_e_par, *src_cdf;
    const int *src_cell, *src_dir_kind, *src_e_kind, *src_group;
};

// Status bits raised by device code (first error wins for the message).
enum DevStatus : int {
    DS_OK = 0,
    DS_OVERFLOW = 3,
    DS_LOST = 4,
    DS_TIMEOUT = 5,
    DS_NAN = 6,
};

constexpr int kNumCounters = 9;   // same order as mc_counters' first fields

// Arguments of the FP64 history kernels.
struct HistoryArgs {
    uint64_t first;          // first history of the chunk
    uint32_t n;              // histories in the chunk
    uint64_t seed;
    double *hist;            // [n][n_bins] per-history totals (scratch)
    void *stack;             // [threads][stack_depth] split particles (scratch)
    uint32_t stack_depth;
    unsigned long long *counters;   // [kNumCounters]
    unsigned long long *digest;     // [n] or nullptr
    int *status;
    unsigned int *next;      // work counter (zeroed by the launcher)
    // likelihood-ratio differentiation (n_params > 0): each history row is
    // followed by n_bins x n_params derivative contributions; split copies
    // keep their score-function weights in lr_stack
    int n_params = 0;
    double *lr_stack = nullptr;   // [threads][stack_depth][n_params]
    // derivative columns per tally bin: the n_params (Sigma_s, Sigma_a) pairs
    // followed by one column per material for rho d/drho (density scales
    // both cross sections of the material)
    int n_cols = 0;
    uint32_t max_events = 1u << 22;   // events per particle before DS_TIMEOUT
};

constexpr int kMaxLrParams = 64;   // (Sigma_s, Sigma_a) for up to 32 materials

// FP64 history-based transport of one chunk.  replay selects the portable
// elementary functions (bit-exact with the CPU oracle); otherwise CUDA's
// native FP64 functions are used.
cudaError_t launch_history_fp64(const DevTables &T, const HistoryArgs &A, bool replay,
                                int grid, int block, cudaStream_t st);

// Folds a chunk's per-history totals into sum / sq.  ordered = history order
// (bit-exact with the reference's end_history loop); otherwise a parallel
// tree fold.
cudaError_t launch_fold(const double *hist, uint32_t n, long long n_bins, double *sum, double *sq,
                        bool ordered, cudaStream_t st);

// Exact per-bin sums (mc_exact.cu): kExactLimbs signed 64-bit limbs per
// value, value = sum_j limb[j] * 2^(32 j - 1074); [n_bins][2][kExactLimbs]
// (sum of history totals, sum of their squares).
constexpr int kExactLimbs = 68;

// Adds a chunk's per-history totals and their squares to ex exactly.
cudaError_t launch_fold_exact(const double *hist, uint32_t n, long long n_bins, long long *ex, cudaStream_t st);

// Propagates the carries of every exact value of ex (one representation per
// value: limbs 0..kExactLimbs-2 in [0, 2^32), the last one signed).
cudaError_t launch_exact_normalize(long long *ex, long long n_bins, cudaStream_t st);

// Bytes of one FP64 split-stack entry.
size_t fp64_particle_bytes();

// Resident-thread estimate for the FP64 history kernel.
int history_fp64_max_threads(bool replay, int block);

}  // namespace mc
