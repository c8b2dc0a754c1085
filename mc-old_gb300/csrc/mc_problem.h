// mc_problem.h -- the fixed-source problem as flat tables.
//
// The reference builds a graph of shared_ptr-linked objects from input.xml
// (src/simulator/setup.cpp:30-1066).  Here the same information is read into
// flat arrays (struct-of-arrays, CSR lists, IDs = input order) that are copied
// to the GPU in one allocation.  Table layouts:
//
//   surfaces   type / bc / 8 coefficients each (see SurfType)
//   cells      importance, material (-1 = void), CSR (surface, sense) lists,
//              CSR lists of attached track-length and collision estimators
//   surfaces   CSR list of attached crossing estimators
//   materials  CSR (nuclide, atom density) lists      -- continuous energy
//              or G-group total / scatter-matrix rows  -- multigroup
//   nuclides   mass A, pointwise grid and sigma_s / sigma_c / sigma_t
//              columns (sigma_t = s + c + f summed at load as setup.cpp:372
//              does), or a constant capture cross section
//   estimators scores (kind, kernel), filters (kind, bins, grid), index
//              factors (Estimator.cpp:280-295), offset into the flat tallies
//   sources    point sources: position, cell, direction / energy sampling
//              parameters, multigroup source group, equal-step CDF
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace mc {

enum SurfType : int32_t { S_PX = 0, S_PY, S_PZ, S_PLANE, S_SPHERE, S_CYLX, S_CYLY, S_CYLZ };
enum Kernel : int32_t { K_TL = 0, K_C = 1, K_NEUTRON = 2 };
enum ScoreKind : int32_t { SC_FLUX = 0, SC_ABSORPTION, SC_SCATTER, SC_CAPTURE, SC_TOTAL };
enum FilterKind : int32_t { F_SURFACE = 0, F_CELL, F_ENERGY, F_TIME, F_GROUP };
enum DirKind : int32_t { D_DELTA = 0, D_ISO, D_XYZ, D_HEMI_X };
enum ScalarKind : int32_t { E_DELTA = 0, E_UNIFORM = 1 };
enum NucKind : int32_t { N_TABLE = 0, N_CONST = 1 };

struct Tables {
    std::string name;
    uint64_t nsample = 0;
    double wr = 0.001, ws = 1.0;
    int32_t comb_bank_max = 0, comb_teeth = 0;   // particle comb (0 teeth: off)

    std::vector<int32_t> surf_type, surf_bc;
    std::vector<double> surf_coef;
    std::vector<std::string> surf_names;

    std::vector<double> cell_imp;
    std::vector<int32_t> cell_mat, cell_surf_off, cell_surf, cell_sense;
    std::vector<int32_t> cell_tl_off, cell_tl, cell_c_off, cell_c, surf_est_off, surf_est;
    std::vector<std::string> cell_names;

    std::vector<int32_t> mat_off, mat_nuc;
    std::vector<double> mat_dens;
    std::vector<std::string> mat_names;

    std::vector<int32_t> nuc_kind, nuc_len;
    std::vector<double> nuc_A, nuc_const;
    std::vector<int64_t> nuc_off;
    std::vector<double> xs_E, xs_S, xs_C, xs_T;

    int32_t mg_groups = 0;
    std::vector<double> mg_total, mg_scatter, mg_scat_tot, mg_capture;

    std::vector<int32_t> est_score_off, score_kind, score_kernel;
    std::vector<int32_t> est_filt_off, filt_kind, filt_size, filt_grid_len;
    std::vector<int64_t> filt_grid_off;
    std::vector<double> filt_grid, est_factor;
    std::vector<int32_t> est_factor_off;
    std::vector<int64_t> est_bin_off;
    std::vector<std::string> est_names;
    std::vector<std::vector<std::string>> est_score_names;

    std::vector<double> src_pos, src_dir_par, src_e_par, src_cdf;
    std::vector<int32_t> src_cell, src_dir_kind, src_e_kind, src_group;

    int n_surf() const { return (int)surf_type.size(); }
    int n_cell() const { return (int)cell_imp.size(); }
    int n_mat() const { return (int)mat_names.size(); }
    int n_nuc() const { return (int)nuc_kind.size(); }
    int n_est() const { return (int)est_names.size(); }
    int n_src() const { return (int)src_cell.size(); }
    int64_t n_bins() const { return est_bin_off.empty() ? 0 : est_bin_off.back(); }
};

// Reads io_dir/input.xml (xs_dir: directory of <ZAID>.txt tables).  Returns
// false and sets err on any input the reference would reject or that lies
// outside the fixed-source non-multiplying scope.
bool load_problem(const std::string &io_dir, const std::string &xs_dir, Tables &t, std::string &err);

// Surface::eval (Geometry.cpp:29-69), host side.
double surface_eval_host(const Tables &t, int s, const double p[3]);

}  // namespace mc
