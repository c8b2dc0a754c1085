/*
 * mc_oracle.c -- CPU oracle for the fixed-source particle-history path.
 *
 * TEST INFRASTRUCTURE.  This file is the oracle: it restates, in plain C, the
 * reference's algorithm for this path so that the CUDA library can be
 * compared with it.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py may load it.  Each function names the reference lines it
 * follows (paths are relative to the MC-old project root).
 *
 * Differences from the reference, all deliberate and shared with the GPU path:
 *  - Urand() (src/Random.cpp:121-126, a global LCG) is replaced by the Philox
 *    stream of orc_philox.h keyed by (seed, history, particle, event, draw).
 *  - log/exp/sin/cos come from orc_math.h (bit-identical on host and GPU).
 *  - Fission is out of scope: collision() (general.cpp:121-163) skips the
 *    implicit-fission block (general.cpp:135-151), draws nothing for it, and
 *    Sigma_f is identically zero.  The reference itself crashes there for
 *    every non-fissile medium (fixed_source.cpp:15 dereferences a null
 *    nuclide).
 *  - A user-defined capture-only nuclide (setup.cpp:434-462) has
 *    sigma_t = sigma_a = sigma_c and sigma_s = 0; the reference leaves its
 *    total cross section null and crashes in Nuclide::sigmaT (Nuclide.cpp:55).
 *  - A lost particle returns ORC_ERR_LOST instead of std::exit
 *    (general.cpp:31-33).
 * The operand-evaluation order the reference compiles to with g++ (the
 * energy distribution of a point source is sampled before its direction,
 * Source.cpp:124; the z component of an independentXYZ direction first,
 * Distribution.cpp:95; in the free-gas "w1" branch the left log's draw
 * first, Reaction.cpp:55-56) is pinned against the compiled reference in the
 * tests and reproduced here.
 */
#include "mc_oracle.h"
#include "orc_math.h"
#include "orc_philox.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Constants.h:7-13 */
#define ORC_PI        0x1.921fb54442d18p+1
#define ORC_PI_2      (2.0 * ORC_PI)
#define ORC_PI_HALF   (0.5 * ORC_PI)
#define ORC_PI_SQRT   0x1.c5bf891b4ef6ap+0   /* sqrt(PI), correctly rounded */
#define ORC_EPS_F     ((double)FLT_EPSILON)
#define ORC_MAX_F     ((double)FLT_MAX)
#define ORC_MAX_F_LESS (0.9 * ORC_MAX_F)

/* Argument-evaluation order of the compiled reference (see file header). */
#ifndef ORC_SOURCE_ENERGY_FIRST
#define ORC_SOURCE_ENERGY_FIRST 1
#endif
#ifndef ORC_FREEGAS_SECOND_LOG_FIRST
#define ORC_FREEGAS_SECOND_LOG_FIRST 0
#endif

typedef struct {
    double x, y, z;        /* position (cm) */
    double u, v, w;        /* direction */
    double E, E_old;       /* energy (eV) */
    double speed;          /* cm/s */
    double wgt;
    double t, t_old;       /* s */
    int    alive;
    int    cell, cell_old, surf_old;
    int    g;              /* multigroup group */
    uint32_t id;
} orc_particle;

typedef struct {
    orc_particle *v;
    size_t n, cap;
} orc_stack;

/* The reference's per-nuclide grid index (Nuclide::checkE,
 * Nuclide.cpp:18-24) and per-table last value (XSTable::xs, XSec.cpp:9-40),
 * kept for the energy they were computed at.  A hit returns the value the
 * computation would give, so the cache changes no result, only the time. */
typedef struct {
    double E_idx;          /* energy of idx (NaN: none yet) */
    int idx;
    double E_tab[3];       /* per column (t, s, c) */
    double xs_tab[3];
} orc_nuc_cache;

typedef struct {
    const orc_problem *P;
    orc_rng rng;
    orc_nuc_cache *nc;     /* [n_nuc] */
    double *hist;
    uint64_t *cnt;
    uint64_t digest;
    orc_stack bank;
    int status;
} orc_ctx;

static int stack_push(orc_stack *s, const orc_particle *p)
{
    if (s->n == s->cap) {
        size_t nc = s->cap ? 2 * s->cap : 64;
        orc_particle *nv = (orc_particle *)realloc(s->v, nc * sizeof(orc_particle));
        if (!nv) return ORC_ERR_NOMEM;
        s->v = nv; s->cap = nc;
    }
    s->v[s->n++] = *p;
    return ORC_OK;
}

static inline void dig(orc_ctx *C, uint64_t v)
{
    C->digest = (C->digest ^ v) * 0x100000001B3ULL;
}

static inline double U(orc_ctx *C) { return orc_urand(&C->rng); }

/* ------------------------------------------------------------------------- */
/* Algorithm.cpp                                                             */
/* ------------------------------------------------------------------------- */

/* Algorithm.cpp:16-38 */
double orc_geometry_quad(double a, double b, double c)
{
    const double D = b * b - 4.0 * a * c;
    if (D <= 0.0) return ORC_MAX_F;
    const double sqrtD = __builtin_sqrt(D);
    const double ai = 0.5 / a;
    double r1 = ai * (-1.0 * b - sqrtD);
    double r2 = ai * (-1.0 * b + sqrtD);
    if (r1 < 0) r1 = ORC_MAX_F;
    if (r2 < 0) r2 = ORC_MAX_F;
    return __builtin_fmin(r1, r2);
}

/* Algorithm.cpp:46-64 */
int orc_binary_search(double x, const double *vec, int n)
{
    int left = 0, right = n - 1, mid;
    while (left <= right) {
        mid = (left + right) / 2;
        if (vec[mid] < x) left = mid + 1;
        else right = mid - 1;
    }
    return right;
}

/* Algorithm.cpp:103-105 */
double orc_interpolate(double x, double x1, double x2, double y1, double y2)
{
    return (x - x2) / (x1 - x2) * y1 + (x - x1) / (x2 - x1) * y2;
}

/* Algorithm.cpp:67-101 */
static void scatter_direction(orc_ctx *C, const double di[3], double mu0, double df[3])
{
    const double azi = ORC_PI_2 * U(C);
    const double cos_azi = orc_cos(azi);
    const double sin_azi = orc_sin(azi);
    const double Ac = __builtin_sqrt(1.0 - mu0 * mu0);
    if (di[2] != 1.0) {
        const double B = __builtin_sqrt(1.0 - di[2] * di[2]);
        const double Cc = Ac / B;
        df[0] = di[0] * mu0 + (di[0] * di[2] * cos_azi - di[1] * sin_azi) * Cc;
        df[1] = di[1] * mu0 + (di[1] * di[2] * cos_azi + di[0] * sin_azi) * Cc;
        df[2] = di[2] * mu0 - cos_azi * Ac * B;
    } else {
        const double B = __builtin_sqrt(1.0 - di[1] * di[1]);
        const double Cc = Ac / B;
        df[0] = di[0] * mu0 + (di[0] * di[1] * cos_azi - di[2] * sin_azi) * Cc;
        df[2] = di[2] * mu0 + (di[2] * di[1] * cos_azi + di[0] * sin_azi) * Cc;
        df[1] = di[1] * mu0 - cos_azi * Ac * B;
    }
}

/* Algorithm.cpp:123-126 */
static double exponential_sample(orc_ctx *C, double param)
{
    return -orc_log(U(C)) / param;
}

/* ------------------------------------------------------------------------- */
/* Particle.cpp                                                              */
/* ------------------------------------------------------------------------- */

/* Particle.cpp:42-48 */
double orc_speed_from_energy(double E) { return 13831.5926439 * __builtin_sqrt(E) * 100.0; }
/* Particle.cpp:49-56 */
double orc_energy_from_speed(double v) { return 5.2270376e-13 * v * v; }

static void p_set_energy(orc_particle *p, double E)
{
    p->E_old = p->E;
    p->E = E;
    p->speed = orc_speed_from_energy(E);
}

static void p_set_speed(orc_particle *p, double v)
{
    p->speed = v;
    p->E_old = p->E;
    p->E = orc_energy_from_speed(v);
}

/* Particle.cpp:66-76 */
static void p_move(orc_particle *p, double d)
{
    p->x += p->u * d;
    p->y += p->v * d;
    p->z += p->w * d;
    p->t_old = p->t;
    p->t += d / p->speed;
}

/* Particle.cpp:77-81 */
static void p_kill(orc_particle *p) { p->alive = 0; p->wgt = 0.0; }

/* Particle.cpp:36-41 */
static void p_set_cell(orc_particle *p, int c) { p->cell_old = p->cell; p->cell = c; }

/* ------------------------------------------------------------------------- */
/* Geometry.cpp                                                              */
/* ------------------------------------------------------------------------- */

/* Geometry.cpp:29-69 */
double orc_surface_eval(const orc_problem *P, int s, const double p[3])
{
    const double *k = P->surf_coef + 8 * (size_t)s;
    switch (P->surf_type[s]) {
    case ORC_PX: return p[0] - k[0];
    case ORC_PY: return p[1] - k[0];
    case ORC_PZ: return p[2] - k[0];
    case ORC_PLANE: return k[0] * p[0] + k[1] * p[1] + k[2] * p[2] - k[3];
    case ORC_SPHERE: {
        const double xt = p[0] - k[0], yt = p[1] - k[1], zt = p[2] - k[2];
        return xt * xt + yt * yt + zt * zt - k[4];
    }
    case ORC_CYLX: {
        const double yt = p[1] - k[0], zt = p[2] - k[1];
        return yt * yt + zt * zt - k[3];
    }
    case ORC_CYLY: {   /* Geometry.cpp:58-63 uses p.y for the z offset */
        const double xt = p[0] - k[0], zt = p[1] - k[1];
        return xt * xt + zt * zt - k[3];
    }
    default: {         /* ORC_CYLZ */
        const double xt = p[0] - k[0], yt = p[1] - k[1];
        return xt * xt + yt * yt - k[3];
    }
    }
}

static double plane_axis_distance(double loc, double pos, double dir)
{
    /* Geometry.cpp:76-126 */
    if (__builtin_fabs(dir) > ORC_EPS_F) {
        const double dist = (loc - pos) / dir;
        if (dist > 0.0) return dist;
        return ORC_MAX_F;
    }
    return ORC_MAX_F;
}

/* Geometry.cpp:76-188 */
double orc_surface_distance(const orc_problem *P, int s, const double p[3], const double u[3])
{
    const double *k = P->surf_coef + 8 * (size_t)s;
    switch (P->surf_type[s]) {
    case ORC_PX: return plane_axis_distance(k[0], p[0], u[0]);
    case ORC_PY: return plane_axis_distance(k[0], p[1], u[1]);
    case ORC_PZ: return plane_axis_distance(k[0], p[2], u[2]);
    case ORC_PLANE: {
        const double denom = k[0] * u[0] + k[1] * u[1] + k[2] * u[2];
        if (__builtin_fabs(denom) > ORC_EPS_F) {
            const double dist = (k[3] - k[0] * p[0] - k[1] * p[1] - k[2] * p[2]) / denom;
            if (dist > 0.0) return dist;
            return ORC_MAX_F;
        }
        return ORC_MAX_F;
    }
    case ORC_SPHERE: {
        const double b = 2.0 * ((p[0] - k[0]) * u[0] + (p[1] - k[1]) * u[1] + (p[2] - k[2]) * u[2]);
        const double c = orc_surface_eval(P, s, p);
        return orc_geometry_quad(1.0, b, c);
    }
    case ORC_CYLX: {
        const double a = 1.0 - u[0] * u[0];
        const double b = 2.0 * ((p[1] - k[0]) * u[1] + (p[2] - k[1]) * u[2]);
        return orc_geometry_quad(a, b, orc_surface_eval(P, s, p));
    }
    case ORC_CYLY: {
        const double a = 1.0 - u[1] * u[1];
        const double b = 2.0 * ((p[0] - k[0]) * u[0] + (p[2] - k[1]) * u[2]);
        return orc_geometry_quad(a, b, orc_surface_eval(P, s, p));
    }
    default: {
        const double a = 1.0 - u[2] * u[2];
        const double b = 2.0 * ((p[0] - k[0]) * u[0] + (p[1] - k[1]) * u[1]);
        return orc_geometry_quad(a, b, orc_surface_eval(P, s, p));
    }
    }
}

/* Geometry.cpp:195-222 (sphere and cylinder reflection are no-ops there) */
void orc_surface_reflect(const orc_problem *P, int s, double u[3])
{
    const double *k = P->surf_coef + 8 * (size_t)s;
    switch (P->surf_type[s]) {
    case ORC_PX: u[0] = -u[0]; break;
    case ORC_PY: u[1] = -u[1]; break;
    case ORC_PZ: u[2] = -u[2]; break;
    case ORC_PLANE: {
        const double K = k[0] * u[0] + k[1] * u[1] + k[2] * u[2];
        const double qx = u[0] - k[4] * K;
        const double qy = u[1] - k[5] * K;
        const double qz = u[2] - k[6] * K;
        u[0] = qx; u[1] = qy; u[2] = qz;
        break;
    }
    default: break;
    }
}

/* ------------------------------------------------------------------------- */
/* XSec.cpp / Nuclide.cpp / Material.cpp                                     */
/* ------------------------------------------------------------------------- */

/* XSec.cpp:9-40 with the bin index from Nuclide::checkE (Nuclide.cpp:18-24),
 * both through the reference's caches (orc_nuc_cache) when c is given. */
static double table_xs(const orc_problem *P, orc_nuc_cache *c, int n, int k, const double *col, double E)
{
    if (c && E == c->E_tab[k]) return c->xs_tab[k];
    const int64_t off = P->nuc_off[n];
    const int len = P->nuc_len[n];
    const double *Eg = P->xs_E + off;
    int idx;
    if (c && E == c->E_idx) {
        idx = c->idx;
    } else {
        idx = orc_binary_search(E, Eg, len);
        if (c) { c->E_idx = E; c->idx = idx; }
    }
    double v;
    if (idx == len - 1) v = col[off + len - 1];
    else if (idx == -1) v = col[off];
    else v = orc_interpolate(E, Eg[idx], Eg[idx + 1], col[off + idx], col[off + idx + 1]);
    if (c) { c->E_tab[k] = E; c->xs_tab[k] = v; }
    return v;
}

enum { XS_T = 0, XS_S, XS_C, XS_A };

static double nuclide_xs(const orc_problem *P, orc_nuc_cache *nc, int n, int which, double E)
{
    if (P->nuc_kind[n] == ORC_NUC_CONST) {
        /* XSec.cpp:5-7; capture-only nuclide: t = a = c, s = 0 */
        return which == XS_S ? 0.0 : P->nuc_const[n];
    }
    orc_nuc_cache *c = nc ? nc + n : NULL;
    switch (which) {
    case XS_T: return table_xs(P, c, n, 0, P->xs_T, E);
    case XS_S: return table_xs(P, c, n, 1, P->xs_S, E);
    default:   return table_xs(P, c, n, 2, P->xs_C, E);   /* c and a (= c + f, f = 0) */
    }
}

/* Material.cpp:18-57: sum over nuclides in input order */
static double macro_xs(orc_ctx *C, int m, int which, const orc_particle *p)
{
    const orc_problem *P = C->P;
    C->cnt[ORC_C_XS_EVALS]++;
    if (P->mg_groups > 0) {
        const int G = P->mg_groups;
        switch (which) {
        case XS_T: return P->mg_total[(size_t)m * G + p->g];
        case XS_S: return P->mg_scat_tot[(size_t)m * G + p->g];
        default:   return P->mg_capture[(size_t)m * G + p->g];
        }
    }
    double sum = 0.0;
    for (int i = P->mat_off[m]; i < P->mat_off[m + 1]; ++i)
        sum += nuclide_xs(P, C->nc, P->mat_nuc[i], which, p->E) * P->mat_dens[i];
    return sum;
}

/* ------------------------------------------------------------------------- */
/* Estimator.cpp                                                             */
/* ------------------------------------------------------------------------- */

typedef struct { int bin; double l; } orc_il;

/* (bin, length) pairs of all filters of one score call; a time filter that
 * spans more bins than fit is reported as ORC_ERR_OVERFLOW (the GPU path has
 * the same fixed budget). */
#define ORC_MAX_FILT 8
#define ORC_MAX_IL 64

/* Filter::idx_l (Estimator.cpp:133-246); writes the pairs to out and returns
 * their number, or -1 when more than cap would be needed. */
static int filter_idx_l(const orc_problem *P, int f, const orc_particle *p, double l,
                        orc_il *out, int cap)
{
    const double *grid = P->filt_grid + P->filt_grid_off[f];
    const int glen = P->filt_grid_len[f];
    const int nbin = glen - 1;
    if (cap < 1) return -1;
    switch (P->filt_kind[f]) {
    case ORC_F_SURFACE: {
        int b = orc_binary_search((double)p->surf_old, grid, glen) + 1;
        if (b < 0 || b >= P->filt_size[f]) return 0;   /* unsorted grids only */
        out[0].bin = b; out[0].l = l; return 1;
    }
    case ORC_F_CELL: {
        int b = orc_binary_search((double)p->cell, grid, glen) + 1;
        if (b < 0 || b >= P->filt_size[f]) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case ORC_F_ENERGY: {
        int b = orc_binary_search(p->E, grid, glen);
        if (b < 0 || b >= nbin) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case ORC_F_GROUP:
        out[0].bin = p->g; out[0].l = l; return 1;
    default: { /* ORC_F_TIME, Estimator.cpp:199-246 */
        const int loc1 = orc_binary_search(p->t_old, grid, glen);
        const int loc2 = orc_binary_search(p->t, grid, glen);
        int n = 0;
        if (loc1 == loc2) {
            if (loc1 >= 0 && loc1 < nbin) { out[0].bin = loc1; out[0].l = l; return 1; }
            return 0;
        }
        const int num_bin = loc2 - loc1 - 1;
        const int need = (loc1 >= 0) + (num_bin > 0 ? num_bin : 0) + (loc2 < nbin);
        if (need > cap) return -1;
        if (loc1 >= 0) {
            out[n].bin = loc1; out[n].l = (grid[loc1 + 1] - p->t_old) * p->speed; ++n;
        }
        for (int i = 1; i <= num_bin; ++i) {
            out[n].bin = loc1 + i; out[n].l = (grid[loc1 + i + 1] - grid[loc1 + i]) * p->speed; ++n;
        }
        if (loc2 < nbin) {
            out[n].bin = loc2; out[n].l = (p->t - grid[loc2]) * p->speed; ++n;
        }
        return n;
    }
    }
}

/* Score::score (Estimator.cpp:17-124) */
static double score_value(orc_ctx *C, int sc, const orc_particle *p, double l)
{
    const orc_problem *P = C->P;
    const int m = P->cell_mat[p->cell];
    double k;
    switch (P->score_kernel[sc]) {
    case ORC_K_TL: k = p->wgt * l; break;
    case ORC_K_C:  k = p->wgt / (m >= 0 ? macro_xs(C, m, XS_T, p) : 0.0); break;
    default:       k = p->wgt; break;
    }
    switch (P->score_kind[sc]) {
    case ORC_S_FLUX:       return k;
    case ORC_S_ABSORPTION: return (m >= 0 ? macro_xs(C, m, XS_A, p) : 0.0) * k;
    case ORC_S_SCATTER:    return (m >= 0 ? macro_xs(C, m, XS_S, p) : 0.0) * k;
    case ORC_S_CAPTURE:    return (m >= 0 ? macro_xs(C, m, XS_C, p) : 0.0) * k;
    default:               return (m >= 0 ? macro_xs(C, m, XS_T, p) : 0.0) * k;
    }
}

/* Estimator::score (Estimator.cpp:298-336) */
static void estimator_score(orc_ctx *C, int e, const orc_particle *p, double l_in)
{
    const orc_problem *P = C->P;
    const int f0 = P->est_filt_off[e], nf = P->est_filt_off[e + 1] - f0;
    const int s0 = P->est_score_off[e], ns = P->est_score_off[e + 1] - s0;
    const double *fac = P->est_factor + P->est_factor_off[e];
    double *hist = C->hist + P->est_bin_off[e];
    if (!(__builtin_fabs(l_in) <= DBL_MAX)) {   /* the loop below would never advance */
        C->status = ORC_ERR_NAN;
        return;
    }
    orc_il il[ORC_MAX_IL];
    int off[ORC_MAX_FILT + 1], nil[ORC_MAX_FILT], idx[ORC_MAX_FILT];
    off[0] = 0;
    for (int i = 0; i < nf; ++i) {
        const int n = filter_idx_l(P, f0 + i, p, l_in, il + off[i], ORC_MAX_IL - off[i]);
        if (n < 0) { C->status = ORC_ERR_OVERFLOW; return; }
        if (n == 0) return;
        nil[i] = n;
        off[i + 1] = off[i] + n;
        idx[i] = 0;
    }
    for (int guard = 0; guard <= off[nf]; ++guard) {   /* each pass advances one filter */
        double l = ORC_MAX_F;
        for (int i = 0; i < nf; ++i) {          /* l = std::min(l, x) */
            const double x = il[off[i] + idx[i]].l;
            l = (x < l) ? x : l;
        }
        int idx1 = 0;
        for (int i = 0; i < nf; ++i) idx1 += (int)(il[off[i] + idx[i]].bin * fac[i + 1]);
        for (int s = 0; s < ns; ++s) {
            hist[idx1] += score_value(C, s0 + s, p, l);
            C->cnt[ORC_C_TALLY_UPDATES]++;
            idx1 += (int)fac[0];
        }
        for (int i = 0; i < nf; ++i) {
            orc_il *cur = &il[off[i] + idx[i]];
            cur->l -= l;
            if (cur->l < ORC_EPS_F) {
                if (idx[i] == nil[i] - 1) return;
                idx[i]++;
            }
        }
        if (nf == 0) return;
    }
}

/* Estimator::end_cycle / end_simulation (Estimator.cpp:347-367), one cycle */
void orc_finalize(const double *sum, const double *sq, int64_t n_bins, uint64_t nsample,
                  double *mean, double *uncer)
{
    const double N = (double)nsample;
    for (int64_t b = 0; b < n_bins; ++b) {
        const double m = sum[b] / N;
        const double us = (sq[b] / N - m * m) / (N - 1.0);
        double tm = 0.0 + m, tu = 0.0 + us;
        mean[b] = tm / 1.0;
        uncer[b] = __builtin_sqrt(tu) / 1.0;
    }
}

/* ------------------------------------------------------------------------- */
/* simulator/general.cpp, population_control.cpp                             */
/* ------------------------------------------------------------------------- */

/* general.cpp:13-20 */
static int test_point(const orc_problem *P, const double p[3], int c)
{
    for (int i = P->cell_surf_off[c]; i < P->cell_surf_off[c + 1]; ++i)
        if (orc_surface_eval(P, P->cell_surf[i], p) * P->cell_sense[i] < 0) return 0;
    return 1;
}

/* general.cpp:26-34 */
static int search_cell(const orc_problem *P, const double p[3])
{
    for (int c = 0; c < P->n_cell; ++c)
        if (test_point(P, p, c)) return c;
    return -1;
}

/* population_control.cpp:9-15 */
static void weight_roulette(orc_ctx *C, orc_particle *p)
{
    if (p->wgt < C->P->wr) {
        if (U(C) < p->wgt / C->P->ws) p->wgt = C->P->ws;
        else p_kill(p);
    }
}

/* population_control.cpp:21-49 */
static void cell_importance(orc_ctx *C, orc_particle *p)
{
    const orc_problem *P = C->P;
    const double Iold = P->cell_imp[p->cell_old];
    const double Inew = P->cell_imp[p->cell];
    if (Inew == Iold) return;
    const double rat = Inew / Iold;
    if (rat < 1.0) {
        if (U(C) < rat) p->wgt = p->wgt / rat;
        else p_kill(p);
    } else {
        const int n = (int)__builtin_floor(rat + U(C));
        p->wgt = p->wgt / (double)n;
        for (int i = 0; i < n - 1; ++i) {
            orc_particle q = *p;
            q.id = orc_child_id(p->id, C->rng.event, (uint32_t)(i + 1));
            if (stack_push(&C->bank, &q) != ORC_OK) { C->status = ORC_ERR_NOMEM; return; }
            C->cnt[ORC_C_SPLITS]++;
        }
    }
}

/* general.cpp:73-83 */
static void move_particle(orc_ctx *C, orc_particle *p, double l)
{
    const orc_problem *P = C->P;
    p_move(p, l);
    C->cnt[ORC_C_FLIGHTS]++;
    const int m = P->cell_mat[p->cell];
    if (m >= 0 && P->mg_groups == 0) C->cnt[ORC_C_NUC_LOOKUPS] += (uint64_t)(P->mat_off[m + 1] - P->mat_off[m]);
    for (int i = P->cell_tl_off[p->cell]; i < P->cell_tl_off[p->cell + 1]; ++i)
        estimator_score(C, P->cell_tl[i], p, l);
}

/* general.cpp:89-115 */
static void surface_hit(orc_ctx *C, orc_particle *p, int s)
{
    const orc_problem *P = C->P;
    C->cnt[ORC_C_CROSSINGS]++;
    p->surf_old = s;
    const int bc = P->surf_bc[s];
    if (bc == 0) {
        p_move(p, ORC_EPS_F);
        const double pos[3] = { p->x, p->y, p->z };
        const int c = search_cell(P, pos);
        if (c < 0) { C->status = ORC_ERR_LOST; p_kill(p); return; }
        p_set_cell(p, c);
    } else if (bc == -1) {
        p_kill(p);
        p_set_cell(p, p->cell);
    } else {
        double d[3] = { p->u, p->v, p->w };
        orc_surface_reflect(P, s, d);
        p->u = d[0]; p->v = d[1]; p->w = d[2];
        p_move(p, ORC_EPS_F);
        p_set_cell(p, p->cell);
    }
    for (int i = P->surf_est_off[s]; i < P->surf_est_off[s + 1]; ++i)
        estimator_score(C, P->surf_est[i], p, 0.0);
    cell_importance(C, p);
}

/* Reaction.cpp:27-118: free-gas elastic scatter, isotropic in the CM frame */
static void free_gas_scatter(orc_ctx *C, orc_particle *p, double A)
{
    const double mu0 = 2.0 * U(C) - 1.0;                  /* Distribution.cpp:74-77 */
    double V_tilda, mu_tilda;
    const double beta = __builtin_sqrt(2.0659834e-11 * A);
    const double y = beta * p->speed;
    for (;;) {
        double x;
        C->cnt[ORC_C_FREEGAS_ITERS]++;
        if (U(C) < 2.0 / (2.0 + ORC_PI_SQRT * y)) {
            const double a = U(C);
            const double b = U(C);
            x = __builtin_sqrt(-orc_log(a * b));
        } else {
            const double cos_arg = ORC_PI_HALF * U(C);
            const double cos_val = orc_cos(cos_arg);
#if ORC_FREEGAS_SECOND_LOG_FIRST
            const double u2 = U(C);
            const double u1 = U(C);
#else
            const double u1 = U(C);
            const double u2 = U(C);
#endif
            x = __builtin_sqrt(-orc_log(u1) - orc_log(u2) * cos_val * cos_val);
        }
        V_tilda = x / beta;
        mu_tilda = 2.0 * U(C) - 1.0;
        const double acc = __builtin_sqrt(p->speed * p->speed + V_tilda * V_tilda
                                          - 2.0 * p->speed * V_tilda * mu_tilda)
                           / (p->speed + V_tilda);
        if (!(U(C) > acc)) break;
    }
    const double dir[3] = { p->u, p->v, p->w };
    double nd[3];
    scatter_direction(C, dir, mu_tilda, nd);
    const double Vl[3] = { nd[0] * V_tilda, nd[1] * V_tilda, nd[2] * V_tilda };
    double vl[3] = { p->speed * p->u, p->speed * p->v, p->speed * p->w };
    const double uc[3] = { (vl[0] + A * Vl[0]) / (1.0 + A),
                           (vl[1] + A * Vl[1]) / (1.0 + A),
                           (vl[2] + A * Vl[2]) / (1.0 + A) };
    double vc[3] = { vl[0] - uc[0], vl[1] - uc[1], vl[2] - uc[2] };
    const double speed_c = __builtin_sqrt(vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]);
    const double dc[3] = { vc[0] / speed_c, vc[1] / speed_c, vc[2] / speed_c };
    double dn[3];
    scatter_direction(C, dc, mu0, dn);
    vc[0] = speed_c * dn[0]; vc[1] = speed_c * dn[1]; vc[2] = speed_c * dn[2];
    vl[0] = vc[0] + uc[0]; vl[1] = vc[1] + uc[1]; vl[2] = vc[2] + uc[2];
    p_set_speed(p, __builtin_sqrt(vl[0] * vl[0] + vl[1] * vl[1] + vl[2] * vl[2]));
    p->u = vl[0] / p->speed; p->v = vl[1] / p->speed; p->w = vl[2] / p->speed;
}

/* general.cpp:121-163 without the implicit-fission block; multigroup media
 * sample the outgoing group from the scatter row the way nuclide_scatter
 * samples a nuclide (Material.cpp:106-115) and scatter isotropically in the
 * lab frame (Distribution.cpp:74-77 then Algorithm.cpp:67-101). */
static void collision(orc_ctx *C, orc_particle *p)
{
    const orc_problem *P = C->P;
    C->cnt[ORC_C_COLLISIONS]++;
    const int m = P->cell_mat[p->cell];
    if (m < 0) { p_kill(p); return; }
    for (int i = P->cell_c_off[p->cell]; i < P->cell_c_off[p->cell + 1]; ++i)
        estimator_score(C, P->cell_c[i], p, 0.0);
    const double implicit = macro_xs(C, m, XS_C, p) + 0.0;
    p->wgt = p->wgt * (macro_xs(C, m, XS_T, p) - implicit) / macro_xs(C, m, XS_T, p);
    if (P->mg_groups > 0) {
        const int G = P->mg_groups;
        const double *row = P->mg_scatter + ((size_t)m * G + p->g) * G;
        const double u = macro_xs(C, m, XS_S, p) * U(C);
        double s = 0.0;
        int gout = -1;
        for (int g2 = 0; g2 < G; ++g2) {
            s += row[g2];
            if (s > u) { gout = g2; break; }
        }
        if (gout < 0) return;
        p->g = gout;
        const double mu = 2.0 * U(C) - 1.0;
        const double d[3] = { p->u, p->v, p->w };
        double nd[3];
        scatter_direction(C, d, mu, nd);
        p->u = nd[0]; p->v = nd[1]; p->w = nd[2];
        return;
    }
    /* Material::nuclide_scatter (Material.cpp:106-115) */
    const double u = macro_xs(C, m, XS_S, p) * U(C);
    double s = 0.0;
    int nuc = -1;
    for (int i = P->mat_off[m]; i < P->mat_off[m + 1]; ++i) {
        s += nuclide_xs(P, C->nc, P->mat_nuc[i], XS_S, p->E) * P->mat_dens[i];
        if (s > u) { nuc = P->mat_nuc[i]; break; }
    }
    if (nuc < 0) return;
    free_gas_scatter(C, p, P->nuc_A[nuc]);
}

static void digest_event(orc_ctx *C, const orc_particle *p, uint64_t type)
{
    dig(C, type | ((uint64_t)(uint32_t)p->cell << 8));
    dig(C, orc_bits(p->x)); dig(C, orc_bits(p->y)); dig(C, orc_bits(p->z));
    dig(C, orc_bits(p->u)); dig(C, orc_bits(p->v)); dig(C, orc_bits(p->w));
    dig(C, C->P->mg_groups > 0 ? (uint64_t)p->g : orc_bits(p->E));
    dig(C, orc_bits(p->wgt));
}

/* general.cpp:177-211 (the time-dependent branch is out of scope) */
static void random_walk(orc_ctx *C, orc_particle *p)
{
    const orc_problem *P = C->P;
    C->rng.id = p->id;
    C->rng.event = 0;
    C->cnt[ORC_C_PARTICLES]++;
    dig(C, 0xA5A5A5A5ULL ^ p->id);
    while (p->alive && C->status == ORC_OK) {
        C->rng.event++;
        C->rng.draw = 0;
        /* general.cpp:54-67 */
        double dist = ORC_MAX_F;
        int S = -1;
        const double pos[3] = { p->x, p->y, p->z };
        const double dir[3] = { p->u, p->v, p->w };
        for (int i = P->cell_surf_off[p->cell]; i < P->cell_surf_off[p->cell + 1]; ++i) {
            const double d = orc_surface_distance(P, P->cell_surf[i], pos, dir);
            if (d < dist) { dist = d; S = P->cell_surf[i]; }
        }
        /* general.cpp:40-48 */
        const int m = P->cell_mat[p->cell];
        const double dcol = (m >= 0) ? exponential_sample(C, macro_xs(C, m, XS_T, p))
                                     : ORC_MAX_F_LESS;
        uint64_t type;
        if (dcol > dist) {
            if (S < 0) { C->status = ORC_ERR_LOST; return; }
            move_particle(C, p, dist);
            surface_hit(C, p, S);
            type = 1;
        } else {
            move_particle(C, p, dcol);
            collision(C, p);
            type = 2;
        }
        weight_roulette(C, p);
        digest_event(C, p, type);
    }
}

/* SourceBank::get_source + SourcePoint::get_source (Source.cpp:20-24,42-45) */
static void sample_source(orc_ctx *C, orc_particle *p)
{
    const orc_problem *P = C->P;
    const double xi = U(C);
    int s = orc_binary_search(xi, P->src_cdf, P->n_src + 1);
    if (s < 0) s = 0;
    if (s >= P->n_src) s = P->n_src - 1;
    const double *dp = P->src_dir_par + 9 * (size_t)s;
    double E = 0.0, d[3];
#if ORC_SOURCE_ENERGY_FIRST
    const int energy_first = 1;
#else
    const int energy_first = 0;
#endif
    for (int pass = 0; pass < 2; ++pass) {
        const int do_energy = (pass == 0) == energy_first;
        if (do_energy) {
            const double *ep = P->src_e_par + 2 * (size_t)s;
            E = (P->src_e_kind[s] == ORC_E_UNIFORM) ? ep[0] + U(C) * ep[1] : ep[0];
        } else {
            switch (P->src_dir_kind[s]) {
            case ORC_D_DELTA: d[0] = dp[0]; d[1] = dp[1]; d[2] = dp[2]; break;
            case ORC_D_ISO: case ORC_D_HEMI_X: {
                /* Distribution.cpp:78-92; the hemisphere variant draws the
                 * cosine to +x uniformly on (0,1) instead of (-1,1) */
                const double mu = (P->src_dir_kind[s] == ORC_D_ISO) ? 2.0 * U(C) - 1.0 : U(C);
                const double azi = ORC_PI_2 * U(C);
                const double c = __builtin_sqrt(1.0 - mu * mu);
                d[1] = orc_cos(azi) * c;
                d[2] = orc_sin(azi) * c;
                d[0] = mu;
                break;
            }
            default: {
                /* DistributionIndepndentXYZ (Distribution.cpp:93-96): the
                 * compiled reference evaluates the z component first */
                for (int k = 2; k >= 0; --k) {
                    const double *q = dp + 3 * k;
                    d[k] = ((int)q[0] == ORC_E_UNIFORM) ? q[1] + U(C) * q[2] : q[1];
                }
                break;
            }
            }
        }
    }
    memset(p, 0, sizeof(*p));
    p->x = P->src_pos[3 * (size_t)s]; p->y = P->src_pos[3 * (size_t)s + 1]; p->z = P->src_pos[3 * (size_t)s + 2];
    p->u = d[0]; p->v = d[1]; p->w = d[2];
    p->alive = 1;
    p->t = 0.0; p->wgt = 1.0;
    p->cell = P->src_cell[s];
    p->cell_old = -1;
    p->surf_old = -1;
    p->E = 0.0;
    p_set_energy(p, E);
    p->g = P->src_group[s];
    p->id = 0;
}

/* Simulator::particle_comb (population_control.cpp:55-84), called after every
 * random walk (handler.cpp:27) on the history's bank.  The one draw (the first
 * tooth) comes from the stream of the particle that just walked, at event
 * ORC_COMB_EVENT.  Every particle passes at most one tooth (the reference's
 * `if`, not a loop), so the comb keeps at most one copy of each particle; the
 * teeth left over keep the bank's first particle with its own weight, as the
 * reference's bank_tmp(comb_teeth, Pbank[0]) does.  Because tooth j is filled
 * from a particle i >= j, the comb compacts the bank in place.  The copies get
 * fresh ids orc_child_id(walker, ORC_COMB_EVENT, j + 1) so that the teeth do
 * not share random streams. */
#define ORC_COMB_EVENT 0xFFFFFFFFu
static void particle_comb(orc_ctx *C, uint32_t walker)
{
    const orc_problem *P = C->P;
    orc_stack *b = &C->bank;
    if (b->n < (size_t)P->comb_bank_max) return;
    double W = 0.0;
    for (size_t i = 0; i < b->n; ++i) W += b->v[i].wgt;
    const double w_avg = W / (double)P->comb_teeth;
    C->rng.id = walker;
    C->rng.event = ORC_COMB_EVENT;
    C->rng.draw = 0;
    double tooth = orc_urand(&C->rng) * w_avg;
    const orc_particle first = b->v[0];
    const size_t teeth = (size_t)P->comb_teeth;
    double sum = 0.0;
    size_t j = 0;
    for (size_t i = 0; i < b->n; ++i) {
        sum += b->v[i].wgt;
        /* j < teeth: the reference writes past bank_tmp if rounding lets
         * one more tooth fit under the total weight */
        if (sum > tooth && j < teeth) {
            b->v[j] = b->v[i];
            b->v[j].wgt = w_avg;
            tooth += w_avg;
            j++;
        }
    }
    while (b->n < teeth) {   /* grow to the comb's size */
        if (stack_push(b, &first) != ORC_OK) { C->status = ORC_ERR_NOMEM; return; }
    }
    for (size_t k = j; k < teeth; ++k) b->v[k] = first;
    b->n = teeth;
    for (size_t k = 0; k < teeth; ++k) b->v[k].id = orc_child_id(walker, ORC_COMB_EVENT, (uint32_t)(k + 1));
    C->cnt[ORC_C_COMBS]++;
}

int64_t orc_n_bins(const orc_problem *P) { return P->est_bin_off[P->n_est]; }

/* Simulator::start for one cycle (handler.cpp:11-48) over a history range */
int orc_run(const orc_problem *P, uint64_t first, uint64_t n, uint64_t seed,
            double *sum, double *sq, uint64_t *counters, uint64_t *digest,
            double *hist_out)
{
    const int64_t nb = orc_n_bins(P);
    orc_ctx C;
    memset(&C, 0, sizeof(C));
    C.P = P;
    C.cnt = counters;
    C.hist = (double *)calloc((size_t)(nb > 0 ? nb : 1), sizeof(double));
    C.nc = (orc_nuc_cache *)malloc((size_t)(P->n_nuc > 0 ? P->n_nuc : 1) * sizeof(orc_nuc_cache));
    if (!C.hist || !C.nc) { free(C.hist); free(C.nc); return ORC_ERR_NOMEM; }
    for (int i = 0; i < P->n_nuc; ++i) {
        C.nc[i].E_idx = NAN;
        C.nc[i].idx = 0;
        for (int k = 0; k < 3; ++k) { C.nc[i].E_tab[k] = NAN; C.nc[i].xs_tab[k] = 0.0; }
    }
    C.rng.seed = seed;
    for (uint64_t h = 0; h < n && C.status == ORC_OK; ++h) {
        C.rng.history = first + h;
        C.rng.id = 0;
        C.rng.event = 0;
        C.rng.draw = 0;
        C.digest = 0xCBF29CE484222325ULL;
        orc_particle p;
        sample_source(&C, &p);
        C.bank.n = 0;
        if (stack_push(&C.bank, &p) != ORC_OK) { C.status = ORC_ERR_NOMEM; break; }
        while (C.bank.n > 0 && C.status == ORC_OK) {
            orc_particle q = C.bank.v[--C.bank.n];
            random_walk(&C, &q);
            if (P->comb_teeth > 0 && C.status == ORC_OK) particle_comb(&C, q.id);
        }
        if (digest) digest[h] = C.digest;
        if (hist_out) memcpy(hist_out + h * (size_t)nb, C.hist, (size_t)nb * sizeof(double));
        for (int64_t b = 0; b < nb; ++b) {   /* Estimator.cpp:339-346 */
            sum[b] += C.hist[b];
            sq[b] += C.hist[b] * C.hist[b];
            C.hist[b] = 0.0;
        }
    }
    free(C.hist);
    free(C.nc);
    free(C.bank.v);
    return C.status;
}

/* exported primitives for the known-answer tests */
double orc_log_(double x) { return orc_log(x); }
double orc_exp_(double x) { return orc_exp(x); }
double orc_sin_(double x) { return orc_sin(x); }
double orc_cos_(double x) { return orc_cos(x); }
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    orc_philox4x32_10(ctr, key, out);
}

/* Random.cpp:121-126 (MCNP 63-bit LCG, generator 5), kept to pin the
 * reference's own known-answer table (Random.cpp:111-117). */
double orc_lcg_next(uint64_t *seed)
{
    *seed = (3512401965023503517ULL * *seed) & (~0ULL >> 1);
    return (double)(*seed * (1.0 / (double)(1ULL << 63)));
}

/* Random.cpp:130-149 */
uint64_t orc_lcg_skip(uint64_t seed, int64_t nskip_in)
{
    const uint64_t mask = ~0ULL >> 1, period = 1ULL << 61;
    int64_t nskip = nskip_in;
    while (nskip < 0) nskip += (int64_t)period;
    uint64_t ns = (uint64_t)nskip & mask;
    uint64_t gen = 1, g = 3512401965023503517ULL, inc = 0, c = 0;
    for (; ns; ns >>= 1) {
        if (ns & 1) { gen = gen * g & mask; inc = (inc * g + c) & mask; }
        c = (g * c + c) & mask;
        g = g * g & mask;
    }
    return (gen * seed + inc) & mask;
}
