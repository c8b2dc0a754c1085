// mc_evtables.cpp -- builds the FP32 event-engine tables (see mc_evtables.h).
#include "mc_evtables.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

namespace mc {

namespace {

struct Pack {
    EvHost &h;
    template <class T>
    void add(const std::vector<T> &v, const T **slot)
    {
        size_t off = (h.blob.size() + 255) & ~(size_t)255;
        h.blob.resize(off + std::max<size_t>(v.size() * sizeof(T), 16), 0);
        if (!v.empty()) std::memcpy(h.blob.data() + off, v.data(), v.size() * sizeof(T));
        h.fix.emplace_back(reinterpret_cast<const void **>(slot), off);
    }
};

template <class A, class B>
std::vector<B> cast(const std::vector<A> &v)
{
    return std::vector<B>(v.begin(), v.end());
}

// Nuclide cross section at E exactly as XSTable::xs does (XSec.cpp:9-40).
double nuc_xs(const Tables &t, int n, const std::vector<double> &col, double E)
{
    if (t.nuc_kind[n] == N_CONST) return &col == &t.xs_S ? 0.0 : t.nuc_const[n];
    const int64_t off = t.nuc_off[n];
    const int len = t.nuc_len[n];
    const double *Eg = &t.xs_E[off];
    int left = 0, right = len - 1;
    while (left <= right) {
        const int mid = (left + right) / 2;
        if (Eg[mid] < E) left = mid + 1;
        else right = mid - 1;
    }
    const int idx = right;
    if (idx == len - 1) return col[off + len - 1];
    if (idx == -1) return col[off];
    const double x1 = Eg[idx], x2 = Eg[idx + 1], y1 = col[off + idx], y2 = col[off + idx + 1];
    return (E - x2) / (x1 - x2) * y1 + (E - x1) / (x2 - x1) * y2;
}

}  // namespace

bool build_event_tables(const Tables &t, EvHost &h, std::string &err)
{
    h = EvHost();
    Pack P{h};
    EvTables &V = h.view;

    // ---- geometry ----
    V.n_surf = t.n_surf();
    V.n_cell = t.n_cell();
    P.add(t.surf_type, &V.surf_type);
    P.add(t.surf_bc, &V.surf_bc);
    std::vector<float> surf_coef = cast<double, float>(t.surf_coef);
    P.add(surf_coef, &V.surf_coef);
    std::vector<float> cimp = cast<double, float>(t.cell_imp);
    P.add(cimp, &V.cell_imp);
    P.add(t.cell_mat, &V.cell_mat);
    P.add(t.cell_surf_off, &V.cell_surf_off);
    P.add(t.cell_surf, &V.cell_surf);
    P.add(t.cell_sense, &V.cell_sense);
    std::vector<std::vector<int>> nb(2 * (size_t)t.n_surf());
    for (int c = 0; c < t.n_cell(); ++c)
        for (int i = t.cell_surf_off[c]; i < t.cell_surf_off[c + 1]; ++i) {
            auto &lst = nb[2 * (size_t)t.cell_surf[i] + (t.cell_sense[i] > 0 ? 1 : 0)];
            if (lst.empty() || lst.back() != c) lst.push_back(c);
        }
    std::vector<int> nb_off(1, 0), nb_cell;
    for (auto &l : nb) {
        nb_cell.insert(nb_cell.end(), l.begin(), l.end());
        nb_off.push_back((int)nb_cell.size());
    }
    P.add(nb_off, &V.nb_off);
    P.add(nb_cell, &V.nb_cell);
    P.add(t.cell_tl_off, &V.cell_tl_off); P.add(t.cell_tl, &V.cell_tl);
    P.add(t.cell_c_off, &V.cell_c_off); P.add(t.cell_c, &V.cell_c);
    P.add(t.surf_est_off, &V.surf_est_off); P.add(t.surf_est, &V.surf_est);

    // ---- estimators ----
    V.n_est = t.n_est();
    V.n_bins = t.n_bins();
    if (t.n_bins() > (1LL << 30)) { err = "too many tally bins"; return false; }
    P.add(t.est_score_off, &V.est_score_off); P.add(t.score_kind, &V.score_kind);
    P.add(t.score_kernel, &V.score_kernel); P.add(t.est_filt_off, &V.est_filt_off);
    P.add(t.filt_kind, &V.filt_kind); P.add(t.filt_size, &V.filt_size);
    P.add(t.filt_grid_len, &V.filt_grid_len);
    std::vector<int> fgo = cast<int64_t, int>(t.filt_grid_off);
    P.add(fgo, &V.filt_grid_off);
    std::vector<float> fg = cast<double, float>(t.filt_grid);
    P.add(fg, &V.filt_grid);
    std::vector<int> fac;
    for (double f : t.est_factor) fac.push_back((int)f);
    P.add(fac, &V.est_factor);
    P.add(t.est_factor_off, &V.est_factor_off);
    std::vector<int> ebo = cast<int64_t, int>(t.est_bin_off);
    P.add(ebo, &V.est_bin_off);
    V.has_time = 0;
    for (int k : t.filt_kind) if (k == F_TIME) V.has_time = 1;
    // the index part of the filter an attachment fixes: the device searches
    // FP32 grids with the id converted to float, so the same search is done
    // here on the same values
    auto fixed_part = [&](int e, int kind, int id) -> int {
        int idx = 0;
        for (int f = t.est_filt_off[e]; f < t.est_filt_off[e + 1]; ++f) {
            if (t.filt_kind[f] != kind) continue;
            const int i = f - t.est_filt_off[e];
            const double *g = &t.filt_grid[t.filt_grid_off[f]];
            const int n = t.filt_grid_len[f];
            int left = 0, right = n - 1;
            const float x = (float)id;
            while (left <= right) {
                const int mid = (left + right) >> 1;
                if ((float)g[mid] < x) left = mid + 1;
                else right = mid - 1;
            }
            const int b = right + 1;
            if (b < 0 || b >= t.filt_size[f]) return -1;
            idx += b * (int)t.est_factor[t.est_factor_off[e] + i + 1];
        }
        return idx;
    };
    std::vector<int> tl_pre(t.cell_tl.size()), c_pre(t.cell_c.size()), s_pre(t.surf_est.size());
    for (int c = 0; c < t.n_cell(); ++c) {
        for (int i = t.cell_tl_off[c]; i < t.cell_tl_off[c + 1]; ++i) tl_pre[i] = fixed_part(t.cell_tl[i], F_CELL, c);
        for (int i = t.cell_c_off[c]; i < t.cell_c_off[c + 1]; ++i) c_pre[i] = fixed_part(t.cell_c[i], F_CELL, c);
    }
    for (int sf = 0; sf < t.n_surf(); ++sf)
        for (int i = t.surf_est_off[sf]; i < t.surf_est_off[sf + 1]; ++i)
            s_pre[i] = fixed_part(t.surf_est[i], F_SURFACE, sf);
    P.add(tl_pre, &V.cell_tl_pre);
    P.add(c_pre, &V.cell_c_pre);
    P.add(s_pre, &V.surf_est_pre);

    // ---- continuous-energy materials ----
    V.n_mat = t.n_mat();
    V.G = t.mg_groups;
    std::vector<int> mgrid_off, mgrid_len, mnuc_off(1, 0), mnuc_id, mnuc_tab, bkt_off, bkt_n, bkt;
    std::vector<float> xrow, nucS, bkt_lo, bkt_inv;
    if (t.mg_groups == 0) {
        for (int m = 0; m < t.n_mat(); ++m) {
            std::vector<double> grid;
            for (int i = t.mat_off[m]; i < t.mat_off[m + 1]; ++i) {
                const int n = t.mat_nuc[i];
                if (t.nuc_kind[n] == N_TABLE)
                    grid.insert(grid.end(), t.xs_E.begin() + t.nuc_off[n], t.xs_E.begin() + t.nuc_off[n] + t.nuc_len[n]);
            }
            std::sort(grid.begin(), grid.end());
            grid.erase(std::unique(grid.begin(), grid.end()), grid.end());
            // grid points that collapse to one float keep only the first
            std::vector<double> g2;
            for (double e : grid)
                if (g2.empty() || (float)e > (float)g2.back()) g2.push_back(e);
            grid.swap(g2);
            if (grid.size() < 2) { grid = {1e-11, 1e11}; }
            if (grid.front() <= 0.0) { err = "non-positive energy grid point"; return false; }
            const int L = (int)grid.size();
            mgrid_off.push_back((int)(xrow.size() / 4));
            mgrid_len.push_back(L);
            for (double e : grid) {
                double sT = 0.0, sS = 0.0, sC = 0.0;
                for (int i = t.mat_off[m]; i < t.mat_off[m + 1]; ++i) {
                    const int n = t.mat_nuc[i];
                    sT += nuc_xs(t, n, t.xs_T, e) * t.mat_dens[i];
                    sS += nuc_xs(t, n, t.xs_S, e) * t.mat_dens[i];
                    sC += nuc_xs(t, n, t.xs_C, e) * t.mat_dens[i];
                }
                xrow.push_back((float)sT);
                xrow.push_back((float)sS);
                xrow.push_back((float)sC);
                xrow.push_back((float)e);
            }
            for (int i = t.mat_off[m]; i < t.mat_off[m + 1]; ++i) {
                const int n = t.mat_nuc[i];
                mnuc_id.push_back(n);
                mnuc_tab.push_back((int)nucS.size());
                for (double e : grid) nucS.push_back((float)(nuc_xs(t, n, t.xs_S, e) * t.mat_dens[i]));
            }
            mnuc_off.push_back((int)mnuc_id.size());
            // log-spaced buckets: about one grid point per bucket, at most 2^16
            const double lo = std::log2(grid.front()), hi = std::log2(grid.back());
            const int nbk = std::max(16, std::min(1 << 16, 2 * L));
            const double inv = nbk / std::max(hi - lo, 1e-30);
            bkt_off.push_back((int)bkt.size());
            bkt_n.push_back(nbk);
            bkt_lo.push_back((float)lo);
            bkt_inv.push_back((float)inv);
            int j = 0;
            for (int b = 0; b < nbk; ++b) {
                const double e0 = std::exp2(lo + b / inv);
                while (j + 1 < L && grid[j + 1] <= e0) ++j;
                bkt.push_back(j);
            }
        }
    }
    P.add(mgrid_off, &V.mgrid_off); P.add(mgrid_len, &V.mgrid_len);
    P.add(xrow, reinterpret_cast<const float **>(&V.xrow));
    P.add(mnuc_off, &V.mnuc_off); P.add(mnuc_id, &V.mnuc_id); P.add(mnuc_tab, &V.mnuc_tab);
    P.add(nucS, &V.nucS);
    std::vector<float> A = cast<double, float>(t.nuc_A);
    P.add(A, &V.nuc_A);
    P.add(bkt_off, &V.bkt_off); P.add(bkt_lo, &V.bkt_lo); P.add(bkt_inv, &V.bkt_inv);
    P.add(bkt_n, &V.bkt_n); P.add(bkt, &V.bkt);

    // ---- multigroup ----
    std::vector<float> mgT = cast<double, float>(t.mg_total), mgS = cast<double, float>(t.mg_scat_tot),
                       mgC = cast<double, float>(t.mg_capture), cdf;
    if (t.mg_groups > 0) {
        const int G = t.mg_groups;
        cdf.resize(t.mg_scatter.size());
        for (size_t r = 0; r < t.mg_scatter.size() / G; ++r) {
            double acc = 0.0;
            for (int g2 = 0; g2 < G; ++g2) {
                acc += t.mg_scatter[r * G + g2];
                cdf[r * G + g2] = (float)acc;
            }
        }
        h.mg_bytes = (mgT.size() * 3 + cdf.size()) * sizeof(float);
    }
    P.add(mgT, &V.mg_total); P.add(mgS, &V.mg_scat_tot); P.add(mgC, &V.mg_capture); P.add(cdf, &V.mg_cdf);

    // ---- sources ----
    V.n_src = t.n_src();
    std::vector<float> sp = cast<double, float>(t.src_pos), sdp = cast<double, float>(t.src_dir_par),
                       sep = cast<double, float>(t.src_e_par), scdf = cast<double, float>(t.src_cdf);
    P.add(sp, &V.src_pos); P.add(sdp, &V.src_dir_par); P.add(sep, &V.src_e_par); P.add(scdf, &V.src_cdf);
    P.add(t.src_cell, &V.src_cell); P.add(t.src_dir_kind, &V.src_dir_kind); P.add(t.src_e_kind, &V.src_e_kind);
    P.add(t.src_group, &V.src_group);
    V.wr = (float)t.wr;
    V.ws = (float)t.ws;
    V.comb_bank_max = t.comb_teeth > 0 ? t.comb_bank_max : 0;
    V.comb_teeth = t.comb_teeth > 0 ? t.comb_teeth : 0;
    return true;
}

}  // namespace mc
