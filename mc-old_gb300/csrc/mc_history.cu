// mc_history.cu -- FP64 history-based transport (replay and plain modes).
//
// One thread walks one history at a time, exactly as Simulator::start and
// Simulator::random_walk do on the CPU (src/simulator/handler.cpp:11-48,
// general.cpp:13-211): the particle and its split copies are processed from a
// per-thread LIFO stack, and every tally contribution is added to the
// history's own row of a per-history bin array, in the reference's order.  A
// second kernel folds the rows into sum / sum-of-squares in history order
// (Estimator::end_history, Estimator.cpp:339-346).
//
// Replay mode uses the portable elementary functions of mc_math.cuh and the
// build uses -fmad=false, so every history's event sequence and every tally
// bin equal the CPU oracle's bit for bit.  Plain mode swaps in CUDA's native
// FP64 log/sin/cos and folds with a parallel tree: the plain double-precision
// GPU history path.
//
// Fission is out of scope: collision() skips the implicit-fission block of
// general.cpp:135-151 and Sigma_f is zero.  A capture-only user nuclide has
// sigma_t = sigma_a = sigma_c, sigma_s = 0 (the reference leaves sigma_t
// unset and crashes).
#include <cfloat>

#include "mc_device.h"
#include "mc_math.cuh"

namespace mc {

namespace {

constexpr double kPi = 0x1.921fb54442d18p+1;
constexpr double kPi2 = 2.0 * kPi;
constexpr double kPiHalf = 0.5 * kPi;
constexpr double kPiSqrt = 0x1.c5bf891b4ef6ap+0;
constexpr double kEpsF = (double)FLT_EPSILON;
constexpr double kMaxF = (double)FLT_MAX;
constexpr double kMaxFLess = 0.9 * kMaxF;
constexpr int kMaxFilt = 8;
constexpr int kMaxIl = 64;
constexpr int kMaxParams = kMaxLrParams;

enum { C_FLIGHTS = 0, C_COLL, C_CROSS, C_TALLY, C_PART, C_SPLIT, C_XS, C_FREEGAS, C_NUC };

struct PartD {
    double x, y, z, u, v, w;
    double E, E_old, speed, wgt, t, t_old;
    int cell, cell_old, surf_old, g;
    unsigned id;
    int alive;
};

template <bool R> struct Fn;
template <> struct Fn<true> {
    static __device__ __forceinline__ double log(double x) { return plog(x); }
    static __device__ __forceinline__ double sin(double x) { return psin(x); }
    static __device__ __forceinline__ double cos(double x) { return pcos(x); }
};
template <> struct Fn<false> {
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double sin(double x) { return ::sin(x); }
    static __device__ __forceinline__ double cos(double x) { return ::cos(x); }
};

struct Ctx {
    const DevTables *T;
    Stream rng;
    double *hist;
    unsigned long long cnt[kNumCounters];
    unsigned long long digest;
    PartD *stack;
    int depth;
    int sp;
    int status;
    // likelihood-ratio (differentiation) state, used only by the L kernels:
    // S[k] = d ln(weight x path probability) / d param_k of the particle being
    // walked; split copies keep theirs in lr_stack
    double S[kMaxParams];
    double *lr_stack;
    int K;                 // parameters: (Sigma_s, Sigma_a) per material
    int Kc;                // derivative columns per bin: K, then K/2 density columns
    uint32_t max_events;   // events per particle before DS_TIMEOUT
    long long nb;          // bins; the derivative rows follow the tally row
};

__device__ __forceinline__ void dig(Ctx &C, unsigned long long v)
{
    C.digest = (C.digest ^ v) * 0x100000001B3ULL;
}

// Algorithm.cpp:46-64
__device__ __forceinline__ int bsearch_d(double x, const double *vec, int n)
{
    int left = 0, right = n - 1;
    while (left <= right) {
        const int mid = (left + right) / 2;
        if (vec[mid] < x) left = mid + 1;
        else right = mid - 1;
    }
    return right;
}

// Algorithm.cpp:16-38
__device__ __forceinline__ double geometry_quad(double a, double b, double c)
{
    const double D = b * b - 4.0 * a * c;
    if (D <= 0.0) return kMaxF;
    const double sqrtD = dsqrt(D);
    const double ai = 0.5 / a;
    double r1 = ai * (-1.0 * b - sqrtD);
    double r2 = ai * (-1.0 * b + sqrtD);
    if (r1 < 0) r1 = kMaxF;
    if (r2 < 0) r2 = kMaxF;
    return fmin(r1, r2);
}

// Algorithm.cpp:103-105
__device__ __forceinline__ double interpolate(double x, double x1, double x2, double y1, double y2)
{
    return (x - x2) / (x1 - x2) * y1 + (x - x1) / (x2 - x1) * y2;
}

// Geometry.cpp:29-69
__device__ double surface_eval(const DevTables &T, int s, double px, double py, double pz)
{
    const double *k = T.surf_coef + 8 * s;
    switch (T.surf_type[s]) {
    case 0: return px - k[0];
    case 1: return py - k[0];
    case 2: return pz - k[0];
    case 3: return k[0] * px + k[1] * py + k[2] * pz - k[3];
    case 4: {
        const double xt = px - k[0], yt = py - k[1], zt = pz - k[2];
        return xt * xt + yt * yt + zt * zt - k[4];
    }
    case 5: {
        const double yt = py - k[0], zt = pz - k[1];
        return yt * yt + zt * zt - k[3];
    }
    case 6: {
        const double xt = px - k[0], zt = py - k[1];
        return xt * xt + zt * zt - k[3];
    }
    default: {
        const double xt = px - k[0], yt = py - k[1];
        return xt * xt + yt * yt - k[3];
    }
    }
}

__device__ __forceinline__ double axis_distance(double loc, double pos, double dir)
{
    if (fabs(dir) > kEpsF) {
        const double dist = (loc - pos) / dir;
        if (dist > 0.0) return dist;
        return kMaxF;
    }
    return kMaxF;
}

// Geometry.cpp:76-188
__device__ double surface_distance(const DevTables &T, int s, const PartD &p)
{
    const double *k = T.surf_coef + 8 * s;
    switch (T.surf_type[s]) {
    case 0: return axis_distance(k[0], p.x, p.u);
    case 1: return axis_distance(k[0], p.y, p.v);
    case 2: return axis_distance(k[0], p.z, p.w);
    case 3: {
        const double denom = k[0] * p.u + k[1] * p.v + k[2] * p.w;
        if (fabs(denom) > kEpsF) {
            const double dist = (k[3] - k[0] * p.x - k[1] * p.y - k[2] * p.z) / denom;
            if (dist > 0.0) return dist;
            return kMaxF;
        }
        return kMaxF;
    }
    case 4: {
        const double b = 2.0 * ((p.x - k[0]) * p.u + (p.y - k[1]) * p.v + (p.z - k[2]) * p.w);
        return geometry_quad(1.0, b, surface_eval(T, s, p.x, p.y, p.z));
    }
    case 5: {
        const double a = 1.0 - p.u * p.u;
        const double b = 2.0 * ((p.y - k[0]) * p.v + (p.z - k[1]) * p.w);
        return geometry_quad(a, b, surface_eval(T, s, p.x, p.y, p.z));
    }
    case 6: {
        const double a = 1.0 - p.v * p.v;
        const double b = 2.0 * ((p.x - k[0]) * p.u + (p.z - k[1]) * p.w);
        return geometry_quad(a, b, surface_eval(T, s, p.x, p.y, p.z));
    }
    default: {
        const double a = 1.0 - p.w * p.w;
        const double b = 2.0 * ((p.x - k[0]) * p.u + (p.y - k[1]) * p.v);
        return geometry_quad(a, b, surface_eval(T, s, p.x, p.y, p.z));
    }
    }
}

// Geometry.cpp:195-222
__device__ void surface_reflect(const DevTables &T, int s, PartD &p)
{
    const double *k = T.surf_coef + 8 * s;
    switch (T.surf_type[s]) {
    case 0: p.u = -p.u; break;
    case 1: p.v = -p.v; break;
    case 2: p.w = -p.w; break;
    case 3: {
        const double K = k[0] * p.u + k[1] * p.v + k[2] * p.w;
        const double qx = p.u - k[4] * K, qy = p.v - k[5] * K, qz = p.w - k[6] * K;
        p.u = qx; p.v = qy; p.w = qz;
        break;
    }
    default: break;
    }
}

// Particle.cpp:42-56, 66-81
__device__ __forceinline__ void p_set_energy(PartD &p, double E)
{
    p.E_old = p.E;
    p.E = E;
    p.speed = 13831.5926439 * dsqrt(E) * 100.0;
}
__device__ __forceinline__ void p_set_speed(PartD &p, double v)
{
    p.speed = v;
    p.E_old = p.E;
    p.E = 5.2270376e-13 * v * v;
}
__device__ __forceinline__ void p_move(PartD &p, double d)
{
    p.x += p.u * d;
    p.y += p.v * d;
    p.z += p.w * d;
    p.t_old = p.t;
    p.t += d / p.speed;
}
__device__ __forceinline__ void p_kill(PartD &p) { p.alive = 0; p.wgt = 0.0; }

enum { XS_T = 0, XS_S, XS_C };

// XSec.cpp:9-40 with Nuclide::checkE's bin (Nuclide.cpp:18-24)
__device__ double table_xs(const DevTables &T, int n, const double *col, double E)
{
    const long long off = T.nuc_off[n];
    const int len = T.nuc_len[n];
    const double *Eg = T.xs_E + off;
    const int idx = bsearch_d(E, Eg, len);
    if (idx == len - 1) return col[off + len - 1];
    if (idx == -1) return col[off];
    return interpolate(E, Eg[idx], Eg[idx + 1], col[off + idx], col[off + idx + 1]);
}

__device__ __forceinline__ double nuclide_xs(const DevTables &T, int n, int which, double E)
{
    if (T.nuc_kind[n] == 1) return which == XS_S ? 0.0 : T.nuc_const[n];
    const double *col = which == XS_T ? T.xs_T : (which == XS_S ? T.xs_S : T.xs_C);
    return table_xs(T, n, col, E);
}

// Material.cpp:18-57 (absorption == capture: sigma_f = 0)
__device__ double macro_xs(Ctx &C, int m, int which, const PartD &p)
{
    const DevTables &T = *C.T;
    C.cnt[C_XS]++;
    if (T.mg_groups > 0) {
        const int i = m * T.mg_groups + p.g;
        return which == XS_T ? T.mg_total[i] : (which == XS_S ? T.mg_scat_tot[i] : T.mg_capture[i]);
    }
    double sum = 0.0;
    for (int i = T.mat_off[m]; i < T.mat_off[m + 1]; ++i)
        sum += nuclide_xs(T, T.mat_nuc[i], which, p.E) * T.mat_dens[i];
    return sum;
}

template <bool R>
__device__ __forceinline__ void scatter_direction(Ctx &C, double dx, double dy, double dz, double mu0,
                                                  double &ox, double &oy, double &oz)
{
    // Algorithm.cpp:67-101
    const double azi = kPi2 * C.rng.next();
    const double cos_azi = Fn<R>::cos(azi);
    const double sin_azi = Fn<R>::sin(azi);
    const double Ac = dsqrt(1.0 - mu0 * mu0);
    if (dz != 1.0) {
        const double B = dsqrt(1.0 - dz * dz);
        const double Cc = Ac / B;
        ox = dx * mu0 + (dx * dz * cos_azi - dy * sin_azi) * Cc;
        oy = dy * mu0 + (dy * dz * cos_azi + dx * sin_azi) * Cc;
        oz = dz * mu0 - cos_azi * Ac * B;
    } else {
        const double B = dsqrt(1.0 - dy * dy);
        const double Cc = Ac / B;
        ox = dx * mu0 + (dx * dy * cos_azi - dz * sin_azi) * Cc;
        oz = dz * mu0 + (dz * dy * cos_azi + dx * sin_azi) * Cc;
        oy = dy * mu0 - cos_azi * Ac * B;
    }
}

struct Il { int bin; double l; };

// Filter::idx_l (Estimator.cpp:133-246); -1 when more than cap pairs needed
__device__ int filter_idx_l(const DevTables &T, int f, const PartD &p, double l, Il *out, int cap)
{
    const double *grid = T.filt_grid + T.filt_grid_off[f];
    const int glen = T.filt_grid_len[f];
    const int nbin = glen - 1;
    if (cap < 1) return -1;
    switch (T.filt_kind[f]) {
    case 0: {
        const int b = bsearch_d((double)p.surf_old, grid, glen) + 1;
        if (b < 0 || b >= T.filt_size[f]) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 1: {
        const int b = bsearch_d((double)p.cell, grid, glen) + 1;
        if (b < 0 || b >= T.filt_size[f]) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 2: {
        const int b = bsearch_d(p.E, grid, glen);
        if (b < 0 || b >= nbin) return 0;
        out[0].bin = b; out[0].l = l; return 1;
    }
    case 4:
        out[0].bin = p.g; out[0].l = l; return 1;
    default: {
        const int loc1 = bsearch_d(p.t_old, grid, glen);
        const int loc2 = bsearch_d(p.t, grid, glen);
        if (loc1 == loc2) {
            if (loc1 >= 0 && loc1 < nbin) { out[0].bin = loc1; out[0].l = l; return 1; }
            return 0;
        }
        const int num_bin = loc2 - loc1 - 1;
        const int need = (loc1 >= 0) + (num_bin > 0 ? num_bin : 0) + (loc2 < nbin);
        if (need > cap) return -1;
        int n = 0;
        if (loc1 >= 0) { out[n].bin = loc1; out[n].l = (grid[loc1 + 1] - p.t_old) * p.speed; ++n; }
        for (int i = 1; i <= num_bin; ++i) {
            out[n].bin = loc1 + i; out[n].l = (grid[loc1 + i + 1] - grid[loc1 + i]) * p.speed; ++n;
        }
        if (loc2 < nbin) { out[n].bin = loc2; out[n].l = (p.t - grid[loc2]) * p.speed; ++n; }
        return n;
    }
    }
}

// Score::score (Estimator.cpp:17-124)
__device__ double score_value(Ctx &C, int sc, const PartD &p, double l)
{
    const DevTables &T = *C.T;
    const int m = T.cell_mat[p.cell];
    double k;
    switch (T.score_kernel[sc]) {
    case 0: k = p.wgt * l; break;
    case 1: k = p.wgt / (m >= 0 ? macro_xs(C, m, XS_T, p) : 0.0); break;
    default: k = p.wgt; break;
    }
    switch (T.score_kind[sc]) {
    case 0: return k;
    case 1: return (m >= 0 ? macro_xs(C, m, XS_C, p) : 0.0) * k;
    case 2: return (m >= 0 ? macro_xs(C, m, XS_S, p) : 0.0) * k;
    case 3: return (m >= 0 ? macro_xs(C, m, XS_C, p) : 0.0) * k;
    default: return (m >= 0 ? macro_xs(C, m, XS_T, p) : 0.0) * k;
    }
}

// d(score)/d(Sigma_s), d(score)/d(Sigma_a) of the cell's material when the
// score itself holds a cross section (Estimator.cpp:29, 60-124); 1-group
__device__ __forceinline__ void direct_terms(const Ctx &C, int sc, int m, const PartD &p, double v,
                                             double &ds, double &da)
{
    const DevTables &T = *C.T;
    ds = 0.0;
    da = 0.0;
    if (m < 0) return;
    const int i = m * T.mg_groups + p.g;
    const double st = T.mg_total[i], ss = T.mg_scat_tot[i], sa = T.mg_capture[i];
    const int kind = T.score_kind[sc];
    if (kind == 2 && ss != 0.0) ds += v / ss;
    if ((kind == 1 || kind == 3) && sa != 0.0) da += v / sa;
    if (kind == 4) { ds += v / st; da += v / st; }
    if (T.score_kernel[sc] == 1) { ds -= v / st; da -= v / st; }
}

// Estimator::score (Estimator.cpp:298-336)
template <bool L>
__device__ void estimator_score(Ctx &C, int e, const PartD &p, double l_in)
{
    const DevTables &T = *C.T;
    const int f0 = T.est_filt_off[e], nf = T.est_filt_off[e + 1] - f0;
    const int s0 = T.est_score_off[e], ns = T.est_score_off[e + 1] - s0;
    const double *fac = T.est_factor + T.est_factor_off[e];
    double *hist = C.hist + T.est_bin_off[e];
    if (!(fabs(l_in) <= DBL_MAX)) {   // non-finite track: the loop below would never advance
        C.status = DS_NAN;
        return;
    }
    Il il[kMaxIl];
    int off[kMaxFilt + 1], nil[kMaxFilt], idx[kMaxFilt];
    off[0] = 0;
    for (int i = 0; i < nf; ++i) {
        const int n = filter_idx_l(T, f0 + i, p, l_in, il + off[i], kMaxIl - off[i]);
        if (n < 0) { C.status = DS_OVERFLOW; return; }
        if (n == 0) return;
        nil[i] = n;
        off[i + 1] = off[i] + n;
        idx[i] = 0;
    }
    for (int guard = 0; guard <= off[nf]; ++guard) {   // each pass advances one filter
        double l = kMaxF;
        for (int i = 0; i < nf; ++i) {
            const double x = il[off[i] + idx[i]].l;
            l = (x < l) ? x : l;
        }
        int idx1 = 0;
        for (int i = 0; i < nf; ++i) idx1 += (int)(il[off[i] + idx[i]].bin * fac[i + 1]);
        for (int s = 0; s < ns; ++s) {
            const double v = score_value(C, s0 + s, p, l);
            hist[idx1] += v;
            C.cnt[C_TALLY]++;
            if constexpr (L) {
                // d(contribution)/d(param_k) = v S_k + direct dependence
                double *dh = C.hist + C.nb + (size_t)(T.est_bin_off[e] + idx1) * C.Kc;
                double ds, da;
                direct_terms(C, s0 + s, T.cell_mat[p.cell], p, v, ds, da);
                const int m = T.cell_mat[p.cell];
                for (int mm = 0; mm < C.K / 2; ++mm) {
                    double d_s = v * C.S[2 * mm], d_a = v * C.S[2 * mm + 1];
                    if (mm == m) { d_s += ds; d_a += da; }
                    dh[2 * mm] += d_s;
                    dh[2 * mm + 1] += d_a;
                    // rho d/drho = Sigma_s d/dSigma_s + Sigma_a d/dSigma_a, per history
                    if (C.Kc > C.K) {
                        const int i = mm * T.mg_groups;
                        dh[C.K + mm] += T.mg_scat_tot[i] * d_s + T.mg_capture[i] * d_a;
                    }
                }
            }
            idx1 += (int)fac[0];
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

// population_control.cpp:9-15
__device__ __forceinline__ void weight_roulette(Ctx &C, PartD &p)
{
    const DevTables &T = *C.T;
    if (p.wgt < T.wr) {
        if (C.rng.next() < p.wgt / T.ws) p.wgt = T.ws;
        else p_kill(p);
    }
}

// population_control.cpp:21-49
template <bool L>
__device__ void cell_importance(Ctx &C, PartD &p)
{
    const DevTables &T = *C.T;
    const double Iold = T.cell_imp[p.cell_old];
    const double Inew = T.cell_imp[p.cell];
    if (Inew == Iold) return;
    const double rat = Inew / Iold;
    if (rat < 1.0) {
        if (C.rng.next() < rat) p.wgt = p.wgt / rat;
        else p_kill(p);
    } else {
        const int n = (int)floor(rat + C.rng.next());
        p.wgt = p.wgt / (double)n;
        for (int i = 0; i < n - 1; ++i) {
            if (C.sp >= C.depth) { C.status = DS_OVERFLOW; return; }
            PartD q = p;
            q.id = child_id(p.id, C.rng.event, (uint32_t)(i + 1));
            if constexpr (L)
                for (int k = 0; k < C.K; ++k) C.lr_stack[(size_t)C.sp * C.K + k] = C.S[k];
            C.stack[C.sp++] = q;
            C.cnt[C_SPLIT]++;
        }
    }
}

// general.cpp:26-34 (search_cell with test_point)
__device__ int search_cell(const DevTables &T, double px, double py, double pz)
{
    for (int c = 0; c < T.n_cell; ++c) {
        bool in = true;
        for (int i = T.cell_surf_off[c]; i < T.cell_surf_off[c + 1]; ++i) {
            if (surface_eval(T, T.cell_surf[i], px, py, pz) * T.cell_sense[i] < 0) { in = false; break; }
        }
        if (in) return c;
    }
    return -1;
}

// general.cpp:73-83
template <bool L>
__device__ void move_particle(Ctx &C, PartD &p, double l)
{
    const DevTables &T = *C.T;
    p_move(p, l);
    C.cnt[C_FLIGHTS]++;
    const int m = T.cell_mat[p.cell];
    if (m >= 0 && T.mg_groups == 0) C.cnt[C_NUC] += (unsigned long long)(T.mat_off[m + 1] - T.mat_off[m]);
    if constexpr (L) {
        // the flight's probability carries exp(-Sigma_t l): d/dSigma_s = d/dSigma_a = -l
        if (m >= 0) { C.S[2 * m] -= l; C.S[2 * m + 1] -= l; }
    }
    for (int i = T.cell_tl_off[p.cell]; i < T.cell_tl_off[p.cell + 1]; ++i)
        estimator_score<L>(C, T.cell_tl[i], p, l);
}

// general.cpp:89-115
template <bool L>
__device__ void surface_hit(Ctx &C, PartD &p, int s)
{
    const DevTables &T = *C.T;
    C.cnt[C_CROSS]++;
    p.surf_old = s;
    const int bc = T.surf_bc[s];
    if (bc == 0) {
        p_move(p, kEpsF);
        const int c = search_cell(T, p.x, p.y, p.z);
        if (c < 0) { C.status = DS_LOST; p_kill(p); return; }
        p.cell_old = p.cell;
        p.cell = c;
    } else if (bc == -1) {
        p_kill(p);
        p.cell_old = p.cell;
    } else {
        surface_reflect(T, s, p);
        p_move(p, kEpsF);
        p.cell_old = p.cell;
    }
    for (int i = T.surf_est_off[s]; i < T.surf_est_off[s + 1]; ++i)
        estimator_score<L>(C, T.surf_est[i], p, 0.0);
    cell_importance<L>(C, p);
}

// Reaction.cpp:27-118
template <bool R>
__device__ void free_gas_scatter(Ctx &C, PartD &p, double A)
{
    const double mu0 = 2.0 * C.rng.next() - 1.0;
    double V_tilda, mu_tilda;
    const double beta = dsqrt(2.0659834e-11 * A);
    const double y = beta * p.speed;
    for (int iter = 0;; ++iter) {
        double x;
        C.cnt[C_FREEGAS]++;
        if (iter > (1 << 20)) { C.status = DS_TIMEOUT; return; }   // acceptance is >= ~1/2
        if (C.rng.next() < 2.0 / (2.0 + kPiSqrt * y)) {
            const double a = C.rng.next();
            const double b = C.rng.next();
            x = dsqrt(-Fn<R>::log(a * b));
        } else {
            const double cos_arg = kPiHalf * C.rng.next();
            const double cos_val = Fn<R>::cos(cos_arg);
            const double u1 = C.rng.next();
            const double u2 = C.rng.next();
            x = dsqrt(-Fn<R>::log(u1) - Fn<R>::log(u2) * cos_val * cos_val);
        }
        V_tilda = x / beta;
        mu_tilda = 2.0 * C.rng.next() - 1.0;
        const double acc = dsqrt(p.speed * p.speed + V_tilda * V_tilda - 2.0 * p.speed * V_tilda * mu_tilda)
                           / (p.speed + V_tilda);
        if (!(C.rng.next() > acc)) break;
    }
    double ndx, ndy, ndz;
    scatter_direction<R>(C, p.u, p.v, p.w, mu_tilda, ndx, ndy, ndz);
    const double Vx = ndx * V_tilda, Vy = ndy * V_tilda, Vz = ndz * V_tilda;
    double vx = p.speed * p.u, vy = p.speed * p.v, vz = p.speed * p.w;
    const double ux = (vx + A * Vx) / (1.0 + A);
    const double uy = (vy + A * Vy) / (1.0 + A);
    const double uz = (vz + A * Vz) / (1.0 + A);
    double cx = vx - ux, cy = vy - uy, cz = vz - uz;
    const double speed_c = dsqrt(cx * cx + cy * cy + cz * cz);
    const double dcx = cx / speed_c, dcy = cy / speed_c, dcz = cz / speed_c;
    double nx, ny, nz;
    scatter_direction<R>(C, dcx, dcy, dcz, mu0, nx, ny, nz);
    cx = speed_c * nx; cy = speed_c * ny; cz = speed_c * nz;
    vx = cx + ux; vy = cy + uy; vz = cz + uz;
    p_set_speed(p, dsqrt(vx * vx + vy * vy + vz * vz));
    p.u = vx / p.speed; p.v = vy / p.speed; p.w = vz / p.speed;
}

// general.cpp:121-163 without implicit fission
template <bool R, bool L>
__device__ void collision(Ctx &C, PartD &p)
{
    const DevTables &T = *C.T;
    C.cnt[C_COLL]++;
    const int m = T.cell_mat[p.cell];
    if (m < 0) { p_kill(p); return; }
    for (int i = T.cell_c_off[p.cell]; i < T.cell_c_off[p.cell + 1]; ++i)
        estimator_score<L>(C, T.cell_c[i], p, 0.0);
    if constexpr (L) {
        // collision density Sigma_t times implicit-capture factor Sigma_s/Sigma_t
        // = Sigma_s: d/dSigma_s = 1/Sigma_s, d/dSigma_a = 0 (1 group)
        C.S[2 * m] += 1.0 / T.mg_scat_tot[m * T.mg_groups + p.g];
    }
    const double implicit = macro_xs(C, m, XS_C, p) + 0.0;
    p.wgt = p.wgt * (macro_xs(C, m, XS_T, p) - implicit) / macro_xs(C, m, XS_T, p);
    if (T.mg_groups > 0) {
        const int G = T.mg_groups;
        const double *row = T.mg_scatter + ((size_t)m * G + p.g) * G;
        const double u = macro_xs(C, m, XS_S, p) * C.rng.next();
        double s = 0.0;
        int gout = -1;
        for (int g2 = 0; g2 < G; ++g2) {
            s += row[g2];
            if (s > u) { gout = g2; break; }
        }
        if (gout < 0) return;
        p.g = gout;
        const double mu = 2.0 * C.rng.next() - 1.0;
        double nx, ny, nz;
        scatter_direction<R>(C, p.u, p.v, p.w, mu, nx, ny, nz);
        p.u = nx; p.v = ny; p.w = nz;
        return;
    }
    // Material::nuclide_scatter (Material.cpp:106-115)
    const double u = macro_xs(C, m, XS_S, p) * C.rng.next();
    double s = 0.0;
    int nuc = -1;
    for (int i = T.mat_off[m]; i < T.mat_off[m + 1]; ++i) {
        s += nuclide_xs(T, T.mat_nuc[i], XS_S, p.E) * T.mat_dens[i];
        if (s > u) { nuc = T.mat_nuc[i]; break; }
    }
    if (nuc < 0) return;
    free_gas_scatter<R>(C, p, T.nuc_A[nuc]);
}

__device__ void digest_event(Ctx &C, const PartD &p, unsigned long long type)
{
    dig(C, type | ((unsigned long long)(unsigned)p.cell << 8));
    dig(C, dbits(p.x)); dig(C, dbits(p.y)); dig(C, dbits(p.z));
    dig(C, dbits(p.u)); dig(C, dbits(p.v)); dig(C, dbits(p.w));
    dig(C, C.T->mg_groups > 0 ? (unsigned long long)p.g : dbits(p.E));
    dig(C, dbits(p.wgt));
}

// general.cpp:177-211
template <bool R, bool L>
__device__ void random_walk(Ctx &C, PartD &p, bool digests)
{
    const DevTables &T = *C.T;
    C.rng.id = p.id;
    C.rng.start_event(0);
    C.cnt[C_PART]++;
    if (digests) dig(C, 0xA5A5A5A5ULL ^ p.id);
    while (p.alive && C.status == DS_OK) {
        C.rng.start_event(C.rng.event + 1);
        if (C.rng.event > C.max_events) { C.status = DS_TIMEOUT; return; }   // bounded walk
        double dist = kMaxF;
        int S = -1;
        for (int i = T.cell_surf_off[p.cell]; i < T.cell_surf_off[p.cell + 1]; ++i) {
            const double d = surface_distance(T, T.cell_surf[i], p);
            if (d < dist) { dist = d; S = T.cell_surf[i]; }
        }
        const int m = T.cell_mat[p.cell];
        const double dcol = (m >= 0) ? -Fn<R>::log(C.rng.next()) / macro_xs(C, m, XS_T, p) : kMaxFLess;
        unsigned long long type;
        if (dcol > dist) {
            if (S < 0) { C.status = DS_LOST; return; }
            move_particle<L>(C, p, dist);
            surface_hit<L>(C, p, S);
            type = 1;
        } else {
            move_particle<L>(C, p, dcol);
            collision<R, L>(C, p);
            type = 2;
        }
        weight_roulette(C, p);
        if (digests) digest_event(C, p, type);
    }
}

// population_control.cpp:55-84, after every random walk (handler.cpp:27), on
// the thread's bank.  The first tooth is the one draw, from the stream of the
// particle that just walked at event kCombEvent.  A particle passes at most
// one tooth (the reference's `if`), and tooth j is filled from a bank entry
// i >= j, so the bank is compacted in place; the teeth left over hold the
// bank's first particle with its own weight (bank_tmp(teeth, Pbank[0])).
// The copies get ids child_id(walker, kCombEvent, j + 1).
constexpr uint32_t kCombEvent = 0xFFFFFFFFu;

__device__ void particle_comb(Ctx &C, uint32_t walker)
{
    const DevTables &T = *C.T;
    if (C.sp < T.comb_bank_max) return;
    const int teeth = T.comb_teeth;
    if (teeth > C.depth) { C.status = DS_OVERFLOW; return; }
    double W = 0.0;
    for (int i = 0; i < C.sp; ++i) W += C.stack[i].wgt;
    const double w_avg = W / (double)teeth;
    C.rng.id = walker;
    C.rng.start_event(kCombEvent);
    double tooth = C.rng.next() * w_avg;
    const PartD first = C.stack[0];
    double sum = 0.0;
    int j = 0;
    for (int i = 0; i < C.sp; ++i) {
        sum += C.stack[i].wgt;
        if (sum > tooth && j < teeth) {   // j < teeth: rounding cannot add a tooth
            PartD q = C.stack[i];
            q.wgt = w_avg;
            C.stack[j++] = q;
            tooth += w_avg;
        }
    }
    for (int k = j; k < teeth; ++k) C.stack[k] = first;
    C.sp = teeth;
    for (int k = 0; k < teeth; ++k) C.stack[k].id = child_id(walker, kCombEvent, (uint32_t)(k + 1));
}

// Source.cpp:20-24, 42-45 and Distribution.cpp:30-33, 78-96
template <bool R>
__device__ void sample_source(Ctx &C, PartD &p)
{
    const DevTables &T = *C.T;
    const double xi = C.rng.next();
    int s = bsearch_d(xi, T.src_cdf, T.n_src + 1);
    s = s < 0 ? 0 : (s >= T.n_src ? T.n_src - 1 : s);
    const double *ep = T.src_e_par + 2 * s;
    // the compiled reference samples the energy before the direction
    const double E = (T.src_e_kind[s] == 1) ? ep[0] + C.rng.next() * ep[1] : ep[0];
    const double *dp = T.src_dir_par + 9 * s;
    double d[3];
    const int dk = T.src_dir_kind[s];
    if (dk == 0) {
        d[0] = dp[0]; d[1] = dp[1]; d[2] = dp[2];
    } else if (dk == 1 || dk == 3) {
        const double mu = (dk == 1) ? 2.0 * C.rng.next() - 1.0 : C.rng.next();
        const double azi = kPi2 * C.rng.next();
        const double c = dsqrt(1.0 - mu * mu);
        d[1] = Fn<R>::cos(azi) * c;
        d[2] = Fn<R>::sin(azi) * c;
        d[0] = mu;
    } else {
        for (int k = 2; k >= 0; --k) {   // z component first, as compiled
            const double *q = dp + 3 * k;
            d[k] = ((int)q[0] == 1) ? q[1] + C.rng.next() * q[2] : q[1];
        }
    }
    p.x = T.src_pos[3 * s]; p.y = T.src_pos[3 * s + 1]; p.z = T.src_pos[3 * s + 2];
    p.u = d[0]; p.v = d[1]; p.w = d[2];
    p.alive = 1;
    p.t = 0.0; p.t_old = 0.0; p.wgt = 1.0;
    p.cell = T.src_cell[s];
    p.cell_old = -1;
    p.surf_old = -1;
    p.E = 0.0;
    p_set_energy(p, E);
    p.g = T.src_group[s];
    p.id = 0;
}

template <bool R, bool L>
__global__ void __launch_bounds__(128) k_history_fp64(const DevTables T, const HistoryArgs A)
{
    Ctx C;
    C.T = &T;
    C.depth = (int)A.stack_depth;
    C.max_events = A.max_events;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    C.stack = reinterpret_cast<PartD *>(A.stack) + tid * A.stack_depth;
    C.status = DS_OK;
    for (int i = 0; i < kNumCounters; ++i) C.cnt[i] = 0;
    const long long nb = T.n_bins;
    C.nb = nb;
    C.K = L ? A.n_params : 0;
    C.Kc = L ? (A.n_cols > A.n_params ? A.n_cols : A.n_params) : 0;
    C.lr_stack = L ? A.lr_stack + tid * A.stack_depth * (size_t)A.n_params : nullptr;
    const long long row = L ? nb * (1 + (long long)C.Kc) : nb;
    const bool digests = A.digest != nullptr;
    for (;;) {
        const unsigned hl = atomicAdd(A.next, 1u);
        if (hl >= A.n) break;
        const uint64_t h = A.first + hl;
        C.hist = A.hist + (size_t)hl * row;
        for (long long b = 0; b < row; ++b) C.hist[b] = 0.0;
        C.rng.init(A.seed, h);
        C.digest = 0xCBF29CE484222325ULL;
        PartD p;
        p.E_old = 0.0;
        sample_source<R>(C, p);
        C.sp = 0;
        if constexpr (L)
            for (int k = 0; k < C.K; ++k) C.lr_stack[k] = 0.0;
        C.stack[C.sp++] = p;
        uint32_t walks = 0;
        while (C.sp > 0 && C.status == DS_OK) {
            --C.sp;
            PartD q = C.stack[C.sp];
            if constexpr (L)
                for (int k = 0; k < C.K; ++k) C.S[k] = C.lr_stack[(size_t)C.sp * C.K + k];
            if (++walks > (1u << 24)) { C.status = DS_TIMEOUT; break; }   // bounded history
            random_walk<R, L>(C, q, digests);
            // the derivative kernels refuse combed problems on the host
            if constexpr (!L)
                if (T.comb_teeth > 0 && C.status == DS_OK) particle_comb(C, q.id);
        }
        if (digests) A.digest[hl] = C.digest;
        if (C.status != DS_OK) {
            atomicCAS(A.status, 0, C.status);
            break;
        }
    }
    for (int i = 0; i < kNumCounters; ++i)
        if (C.cnt[i]) atomicAdd(A.counters + i, C.cnt[i]);
}

// one thread per bin, histories in order (Estimator.cpp:339-346)
__global__ void k_fold_ordered(const double *__restrict__ hist, uint32_t n, long long nb,
                               double *__restrict__ sum, double *__restrict__ sq)
{
    const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    double s = sum[b], q = sq[b];
    uint32_t h = 0;
    for (; h + 8 <= n; h += 8) {
        double v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = hist[(size_t)(h + k) * nb + b];
#pragma unroll
        for (int k = 0; k < 8; ++k) { s += v[k]; q += v[k] * v[k]; }
    }
    for (; h < n; ++h) {
        const double v = hist[(size_t)h * nb + b];
        s += v;
        q += v * v;
    }
    sum[b] = s;
    sq[b] = q;
}

// block-tree fold over a tile of histories per block, FP64 atomics per bin
__global__ void k_fold_tree(const double *__restrict__ hist, uint32_t n, long long nb,
                            double *__restrict__ sum, double *__restrict__ sq, uint32_t rows_per_block)
{
    const uint32_t h0 = blockIdx.y * rows_per_block;
    const uint32_t h1 = min(n, h0 + rows_per_block);
    for (long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
         b += (long long)gridDim.x * blockDim.x) {
        double s = 0.0, q = 0.0;
        for (uint32_t h = h0; h < h1; ++h) {
            const double v = hist[(size_t)h * nb + b];
            s += v;
            q += v * v;
        }
        if (s != 0.0 || q != 0.0) {
            atomicAdd(sum + b, s);
            atomicAdd(sq + b, q);
        }
    }
}

}  // namespace

size_t fp64_particle_bytes() { return sizeof(PartD); }

int history_fp64_max_threads(bool replay, int block)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (replay) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_history_fp64<true, false>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_history_fp64<false, false>, block, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm * block;
}

cudaError_t launch_history_fp64(const DevTables &T, const HistoryArgs &A, bool replay, int grid, int block,
                                cudaStream_t st)
{
    if (A.n_params > 0) {
        if (!replay || A.n_params > kMaxParams) return cudaErrorInvalidValue;
        k_history_fp64<true, true><<<grid, block, 0, st>>>(T, A);
    } else if (replay) {
        k_history_fp64<true, false><<<grid, block, 0, st>>>(T, A);
    } else {
        k_history_fp64<false, false><<<grid, block, 0, st>>>(T, A);
    }
    return cudaGetLastError();
}

cudaError_t launch_fold(const double *hist, uint32_t n, long long nb, double *sum, double *sq, bool ordered,
                        cudaStream_t st)
{
    if (nb <= 0 || n == 0) return cudaSuccess;
    if (ordered) {
        const int block = 128;
        const int grid = (int)((nb + block - 1) / block);
        k_fold_ordered<<<grid, block, 0, st>>>(hist, n, nb, sum, sq);
    } else {
        const int block = 128;
        const uint32_t rows = 512;
        dim3 grid((unsigned)((nb + block - 1) / block), (n + rows - 1) / rows);
        k_fold_tree<<<grid, block, 0, st>>>(hist, n, nb, sum, sq, rows);
    }
    return cudaGetLastError();
}

}  // namespace mc
