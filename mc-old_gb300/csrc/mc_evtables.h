// mc_evtables.h -- FP32 tables of the mixed-precision event engine.
//
// Built on the host from Tables (mc_problem.h):
//  * geometry in FP32, plus per-(surface, side) neighbour lists: the cells
//    that list a surface with a given sense, in input order, which is where a
//    particle crossing that surface can land;
//  * continuous-energy data as per-material macroscopic tables on the union
//    of the material's nuclide energy grids.  Each nuclide's cross section is
//    linear between its own grid points, so between consecutive union points
//    every nuclide -- and their density-weighted sum -- is linear: one
//    interpolation of Sigma_t / Sigma_s / Sigma_c replaces the reference's
//    per-nuclide loop (Material.cpp:18-57) with the same values up to
//    rounding.  N_k sigma_s,k per nuclide on the same grid serves the
//    scatter-nuclide choice (Material.cpp:106-115).  A log-spaced bucket
//    table maps log2(E) to a grid index, so no binary search is needed;
//  * multigroup data in FP32 with cumulative scatter rows.
#pragma once

#include <stdint.h>
#include <vector_types.h>   // float4 (plain struct; host code builds the rows)

#include <vector>

#include "mc_problem.h"

namespace mc {

struct EvTables {
    // geometry
    int n_surf, n_cell;
    const int *surf_type, *surf_bc;
    const float *surf_coef;           // 8 per surface
    const float *cell_imp;
    const int *cell_mat, *cell_surf_off, *cell_surf, *cell_sense;
    const int *nb_off, *nb_cell;      // CSR over 2*n_surf lists: index 2*s + (sense > 0)
    const int *cell_tl_off, *cell_tl, *cell_c_off, *cell_c, *surf_est_off, *surf_est;
    // per attachment above: the part of the flattened tally index that the
    // estimator's cell filter (track-length, collision) or surface filter
    // (crossing) contributes, fixed by the attachment; -1 = outside the filter
    const int *cell_tl_pre, *cell_c_pre, *surf_est_pre;
    // estimators
    int n_est;
    long long n_bins;
    const int *est_score_off, *score_kind, *score_kernel;
    const int *est_filt_off, *filt_kind, *filt_size, *filt_grid_len;
    const int *filt_grid_off;
    const float *filt_grid;
    const int *est_factor;            // nfilt+1 per estimator (integers)
    const int *est_factor_off;
    const int *est_bin_off;
    int has_time;                     // a time filter exists (track time)
    // continuous-energy materials
    int n_mat;
    const int *mgrid_off, *mgrid_len; // per material
    // union grid and macroscopic tables, one 16-byte row per grid point:
    // {Sigma_t, Sigma_s, Sigma_c, E}, so that the two rows bracketing E
    // (one 32-byte load) give the bracket check and all three values
    const float4 *xrow;
    const int *mnuc_off;              // per material: first entry in the nuclide lists
    const int *mnuc_id;               // nuclide index (for the mass A)
    const int *mnuc_tab;              // offset of N_k sigma_s,k on the material grid
    const float *nucS;                // N_k sigma_s,k tables
    const float *nuc_A;
    const int *bkt_off;               // per material
    const float *bkt_lo, *bkt_inv;    // log2(E0) and buckets per unit log2
    const int *bkt_n;
    const int *bkt;                   // grid index of the last point <= bucket start
    // multigroup
    int G;
    const float *mg_total, *mg_scat_tot, *mg_capture;   // [n_mat][G]
    const float *mg_cdf;              // [n_mat][G][G] cumulative scatter rows
    // sources
    int n_src;
    const float *src_pos, *src_dir_par, *src_e_par, *src_cdf;
    const int *src_cell, *src_dir_kind, *src_e_kind, *src_group;
    float wr, ws;
    int comb_bank_max, comb_teeth;    // particle comb (0 teeth: off)
};

// Host-side storage behind EvTables (one packed device allocation).
struct EvHost {
    std::vector<char> blob;                     // packed arrays
    std::vector<std::pair<const void **, size_t>> fix;
    EvTables view{};
    size_t mg_bytes = 0;                        // bytes of the MG tables
};

// Builds the FP32 tables; false + err if the problem cannot run in this mode.
bool build_event_tables(const Tables &t, EvHost &h, std::string &err);

}  // namespace mc
