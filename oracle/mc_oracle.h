/*
 * mc_oracle.h -- CPU oracle for the fixed-source particle-history path.
 *
 * TEST INFRASTRUCTURE.  This is the oracle, not the product: only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py load it.  It is
 * a plain-C restatement of the reference's history loop (MC-old,
 * src/simulator/handler.cpp:11-48, src/simulator/general.cpp:13-211) and of
 * the physics, geometry and tally objects it calls, with the reference's
 * global LCG replaced by the Philox stream of orc_philox.h and libm replaced
 * by orc_math.h so that the GPU's FP64 replay mode can be compared bit for bit.
 *
 * The problem arrives as flat arrays (built by oracle/problem.py from the
 * same input.xml the reference reads).  Layout conventions are documented on
 * each field.
 */
#ifndef MC_ORACLE_H
#define MC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_OK = 0, ORC_ERR_INPUT = 1, ORC_ERR_OVERFLOW = 3, ORC_ERR_LOST = 4, ORC_ERR_NAN = 6, ORC_ERR_NOMEM = 7 };

/* surface types; coefficient layout (8 doubles per surface):
 *   PX/PY/PZ : [loc]
 *   PLANE    : [a, b, c, d, modx, mody, modz]      (Geometry.cpp:14-23)
 *   SPHERE   : [x0, y0, z0, r, r*r]
 *   CYLX     : [y0, z0, r, r*r]; CYLY: [x0, z0, r, r*r]; CYLZ: [x0, y0, r, r*r] */
enum { ORC_PX = 0, ORC_PY, ORC_PZ, ORC_PLANE, ORC_SPHERE, ORC_CYLX, ORC_CYLY, ORC_CYLZ };
/* estimator score kernels (Estimator.cpp:17-30) */
enum { ORC_K_TL = 0, ORC_K_C = 1, ORC_K_NEUTRON = 2 };
/* scores (Estimator.cpp:54-124; fission scores are out of scope) */
enum { ORC_S_FLUX = 0, ORC_S_ABSORPTION, ORC_S_SCATTER, ORC_S_CAPTURE, ORC_S_TOTAL };
/* filters (Estimator.cpp:133-246) plus the multigroup group filter */
enum { ORC_F_SURFACE = 0, ORC_F_CELL, ORC_F_ENERGY, ORC_F_TIME, ORC_F_GROUP };
/* source direction distributions (Distribution.cpp:78-96) plus the inward
 * hemisphere (cosine to +x uniform on (0,1)) */
enum { ORC_D_DELTA = 0, ORC_D_ISO, ORC_D_XYZ, ORC_D_HEMI_X };
/* scalar distributions (Distribution.h delta, Distribution.cpp:30-33 uniform) */
enum { ORC_E_DELTA = 0, ORC_E_UNIFORM = 1 };
/* nuclide kinds: pointwise table (setup.cpp:324-432) or the user-defined
 * capture-only constant nuclide (setup.cpp:434-462) */
enum { ORC_NUC_TABLE = 0, ORC_NUC_CONST = 1 };

typedef struct orc_problem {
    /* surfaces */
    int32_t n_surf;
    const int32_t *surf_type;
    const int32_t *surf_bc;        /* 0 transmission, 1 reflective, -1 vacuum */
    const double  *surf_coef;      /* 8 per surface */
    /* cells, in input order (cell ID = index) */
    int32_t n_cell;
    const double  *cell_imp;
    const int32_t *cell_mat;       /* -1: no material (void / graveyard) */
    const int32_t *cell_surf_off;  /* n_cell+1 */
    const int32_t *cell_surf;      /* surface index */
    const int32_t *cell_sense;
    const int32_t *cell_tl_off;    /* n_cell+1: track-length estimators attached */
    const int32_t *cell_tl;
    const int32_t *cell_c_off;     /* n_cell+1: collision estimators attached */
    const int32_t *cell_c;
    const int32_t *surf_est_off;   /* n_surf+1: crossing estimators attached */
    const int32_t *surf_est;
    /* continuous-energy materials: (nuclide, density) lists */
    int32_t n_mat;
    const int32_t *mat_off;        /* n_mat+1 */
    const int32_t *mat_nuc;
    const double  *mat_dens;
    /* nuclides */
    int32_t n_nuc;
    const int32_t *nuc_kind;
    const double  *nuc_A;
    const double  *nuc_const;      /* capture xs of constant nuclides */
    const int64_t *nuc_off;        /* start in the point arrays */
    const int32_t *nuc_len;        /* number of energy points */
    const double  *xs_E;           /* energy grid (eV) */
    const double  *xs_S;           /* sigma_s */
    const double  *xs_C;           /* sigma_c  (== sigma_a, sigma_f = 0) */
    const double  *xs_T;           /* sigma_t = s + c + f, summed at load */
    /* multigroup (mg_groups > 0 replaces the CE data model for every material) */
    int32_t mg_groups;
    const double  *mg_total;       /* [n_mat][G] */
    const double  *mg_scatter;     /* [n_mat][G][G] row g -> g' */
    const double  *mg_scat_tot;    /* [n_mat][G] row sums (left to right) */
    const double  *mg_capture;     /* [n_mat][G] total - scat_tot */
    /* estimators */
    int32_t n_est;
    const int32_t *est_score_off;  /* n_est+1 into score_kind / score_kernel */
    const int32_t *score_kind;
    const int32_t *score_kernel;
    const int32_t *est_filt_off;   /* n_est+1 into filt_* */
    const int32_t *filt_kind;
    const int32_t *filt_size;      /* number of bins */
    const int64_t *filt_grid_off;
    const int32_t *filt_grid_len;
    const double  *filt_grid;
    const double  *est_factor;     /* per estimator: nfilt+1 (Estimator.cpp:280-295) */
    const int32_t *est_factor_off; /* n_est+1 */
    const int64_t *est_bin_off;    /* n_est+1 into the flat tally arrays */
    /* sources (all point sources; picked uniformly, Source.cpp:42-45,65-72) */
    int32_t n_src;
    const double  *src_pos;        /* 3 per source */
    const int32_t *src_cell;
    const int32_t *src_dir_kind;
    const double  *src_dir_par;    /* 9 per source */
    const int32_t *src_e_kind;
    const double  *src_e_par;      /* 2 per source: delta [val], uniform [a, b-a] */
    const int32_t *src_group;
    const double  *src_cdf;        /* n_src+1 equal-step CDF (Source.cpp:65-72) */
    /* population control (simulator.h:90-91 defaults, overridable) */
    double wr, ws;
    /* particle comb (setup.cpp:57-67); comb_teeth == 0: off */
    int32_t comb_bank_max, comb_teeth;
} orc_problem;

/* counters, in order */
enum {
    ORC_C_FLIGHTS = 0,   /* move_particle calls (the reference's Ntrack) */
    ORC_C_COLLISIONS,
    ORC_C_CROSSINGS,
    ORC_C_TALLY_UPDATES, /* hist += score operations */
    ORC_C_PARTICLES,     /* particles walked, secondaries included */
    ORC_C_SPLITS,        /* copies pushed by importance splitting */
    ORC_C_XS_EVALS,      /* macroscopic Sigma_x(E) evaluations */
    ORC_C_FREEGAS_ITERS, /* free-gas rejection-loop iterations */
    ORC_C_NUC_LOOKUPS,   /* sum over flights of the material's nuclide count */
    ORC_C_COMBS,         /* particle-comb passes over the bank */
    ORC_C_N
};

/* Runs histories [first, first+n) in order and folds each history's bin
 * totals into sum / sq (Estimator.cpp:339-346), continuing whatever those
 * arrays hold.  counters (ORC_C_N) are incremented.  digest (nullable, n
 * entries) receives a per-history hash of the event sequence.  hist_out
 * (nullable, n * n_bins) receives each history's bin totals. */
int orc_run(const orc_problem *P, uint64_t first, uint64_t n, uint64_t seed,
            double *sum, double *sq, uint64_t *counters, uint64_t *digest,
            double *hist_out);

/* Total number of tally bins. */
int64_t orc_n_bins(const orc_problem *P);

/* end_cycle / end_simulation for one cycle (Estimator.cpp:347-367). */
void orc_finalize(const double *sum, const double *sq, int64_t n_bins, uint64_t nsample,
                  double *mean, double *uncer);

/* primitives exposed for known-answer tests */
int    orc_binary_search(double x, const double *vec, int n);
double orc_geometry_quad(double a, double b, double c);
double orc_interpolate(double x, double x1, double x2, double y1, double y2);
double orc_surface_distance(const orc_problem *P, int s, const double pos[3], const double dir[3]);
double orc_surface_eval(const orc_problem *P, int s, const double pos[3]);
void   orc_surface_reflect(const orc_problem *P, int s, double dir[3]);
double orc_speed_from_energy(double E);
double orc_energy_from_speed(double v);
double orc_log_(double x);
double orc_exp_(double x);
double orc_sin_(double x);
double orc_cos_(double x);
void   orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t orc_lcg_skip(uint64_t seed, int64_t n);   /* Random.cpp:130-149 */
double orc_lcg_next(uint64_t *seed);                /* Random.cpp:121-126 */

#ifdef __cplusplus
}
#endif
#endif /* MC_ORACLE_H */
