// mc_problem.cpp -- input.xml -> flat tables (see mc_problem.h).
//
// Follows the reference's reader, src/simulator/setup.cpp, section by
// section: description (:42-50), population control (:57-67), distributions
// (:174-305), nuclides (:310-467), materials (:474-492), surfaces (:499-584),
// cells (:591-629), estimators (:637-805), sources (:1020-1066).  Inputs the
// reference accepts but this path does not cover (k-eigenvalue, TDMC, TRMM,
// fission data, particle comb, Watt spectra) are rejected with a message
// instead of running something different.  Schema additions: a
// <weight_roulette wr ws> override, multigroup materials, the inward
// hemisphere direction distribution, a source group, a group filter.
#include "mc_problem.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>

#include "mc_math.cuh"
#include "mc_xml.h"

namespace mc {

namespace {

bool read_file(const std::string &path, std::string &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

std::vector<double> doubles(const std::string &s)
{
    std::vector<double> v;
    std::istringstream iss(s);
    for (double x; iss >> x;) v.push_back(x);
    return v;
}

template <class T>
int index_of(const std::vector<T> &v, const T &x)
{
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i] == x) return (int)i;
    return -1;
}

void offsets_from(const std::vector<std::vector<int32_t>> &lists, std::vector<int32_t> &off,
                  std::vector<int32_t> &flat)
{
    off.assign(lists.size() + 1, 0);
    flat.clear();
    for (size_t i = 0; i < lists.size(); ++i) {
        flat.insert(flat.end(), lists[i].begin(), lists[i].end());
        off[i + 1] = (int32_t)flat.size();
    }
}

struct ScalarDist { int32_t kind; double a, range; };
struct PointDist { int32_t kind; double par[9]; };

}  // namespace

double surface_eval_host(const Tables &t, int s, const double p[3])
{
    const double *k = &t.surf_coef[8 * (size_t)s];
    switch (t.surf_type[s]) {
    case S_PX: return p[0] - k[0];
    case S_PY: return p[1] - k[0];
    case S_PZ: return p[2] - k[0];
    case S_PLANE: return k[0] * p[0] + k[1] * p[1] + k[2] * p[2] - k[3];
    case S_SPHERE: {
        const double xt = p[0] - k[0], yt = p[1] - k[1], zt = p[2] - k[2];
        return xt * xt + yt * yt + zt * zt - k[4];
    }
    case S_CYLX: {
        const double yt = p[1] - k[0], zt = p[2] - k[1];
        return yt * yt + zt * zt - k[3];
    }
    case S_CYLY: {
        const double xt = p[0] - k[0], zt = p[1] - k[1];
        return xt * xt + zt * zt - k[3];
    }
    default: {
        const double xt = p[0] - k[0], yt = p[1] - k[1];
        return xt * xt + yt * yt - k[3];
    }
    }
}

bool load_problem(const std::string &io_dir, const std::string &xs_dir, Tables &t, std::string &err)
{
    t = Tables();
    std::string text;
    const std::string path = io_dir + "/input.xml";
    if (!read_file(path, text)) { err = "cannot read " + path; return false; }
    XmlNode doc;
    if (!xml_parse(text, doc, err)) { err = path + ": " + err; return false; }

    // ---- description (setup.cpp:42-50) ----
    const XmlNode *sim = doc.child("simulation");
    const XmlNode *desc = sim ? sim->child("description") : nullptr;
    if (desc) {
        t.name = desc->as_string("name");
        t.nsample = (uint64_t)desc->as_double("samples");
    }
    if (sim && (sim->child("ksearch") || sim->child("tdmc"))) {
        err = "k-eigenvalue and time-dependent modes are outside the fixed-source path";
        return false;
    }
    if (doc.child("trmm")) { err = "TRMM is outside the fixed-source path"; return false; }

    // ---- population control (setup.cpp:57-67, simulator.h:90-91) ----
    if (const XmlNode *ctrl = doc.child("population_control")) {
        if (const XmlNode *c = ctrl->child("particle_comb")) {
            t.comb_bank_max = (int32_t)c->as_int("bank_max");
            t.comb_teeth = (int32_t)c->as_int("teeth");
            if (t.comb_bank_max < 1 || t.comb_teeth < 1) {
                err = "<particle_comb> needs bank_max >= 1 and teeth >= 1";
                return false;
            }
            // with more teeth than bank_max, the combed bank is still at least
            // bank_max after the next pop and the history never ends
            if (t.comb_teeth > t.comb_bank_max) {
                err = "<particle_comb> teeth > bank_max never empties the bank";
                return false;
            }
        }
        if (const XmlNode *w = ctrl->child("weight_roulette")) {
            t.wr = w->as_double("wr", t.wr);
            t.ws = w->as_double("ws", t.ws);
        }
    }
    const XmlNode *mgnode = doc.child("multigroup");
    const int G = mgnode ? (int)mgnode->as_int("groups") : 0;
    if (mgnode && G <= 0) { err = "<multigroup groups> must be positive"; return false; }
    t.mg_groups = G;

    // ---- distributions (setup.cpp:174-305): resolve until no progress ----
    std::map<std::string, ScalarDist> ddist;
    std::map<std::string, PointDist> pdist;
    if (const XmlNode *dn = doc.child("distributions")) {
        std::vector<const XmlNode *> pending;
        for (const auto &c : dn->children) pending.push_back(&c);
        while (!pending.empty()) {
            std::vector<const XmlNode *> rest;
            bool progressed = false;
            for (const XmlNode *d : pending) {
                const std::string nm = d->as_string("name"), dt = d->as_string("datatype");
                if (dt == "double") {
                    if (ddist.count(nm)) { progressed = true; continue; }
                    if (d->name == "delta") ddist[nm] = {E_DELTA, d->as_double("val"), 0.0};
                    else if (d->name == "uniform") {
                        const double a = d->as_double("a"), b = d->as_double("b");
                        ddist[nm] = {E_UNIFORM, a, b - a};
                    } else { err = "unsupported double distribution " + d->name; return false; }
                    progressed = true;
                } else if (dt == "point") {
                    if (pdist.count(nm)) { progressed = true; continue; }
                    PointDist p{};
                    if (d->name == "delta") {
                        p.kind = D_DELTA;
                        p.par[0] = d->as_double("x"); p.par[1] = d->as_double("y"); p.par[2] = d->as_double("z");
                    } else if (d->name == "isotropic") {
                        p.kind = D_ISO;
                    } else if (d->name == "isotropic_hemisphere") {
                        p.kind = D_HEMI_X;
                    } else if (d->name == "independentXYZ") {
                        const std::string px = d->as_string("x"), py = d->as_string("y"), pz = d->as_string("z");
                        if (!ddist.count(px) || !ddist.count(py) || !ddist.count(pz)) { rest.push_back(d); continue; }
                        p.kind = D_XYZ;
                        const std::string parts[3] = {px, py, pz};
                        for (int k = 0; k < 3; ++k) {
                            const ScalarDist &s = ddist[parts[k]];
                            p.par[3 * k] = (double)s.kind; p.par[3 * k + 1] = s.a; p.par[3 * k + 2] = s.range;
                        }
                    } else { err = "unsupported point distribution " + d->name; return false; }
                    pdist[nm] = p;
                    progressed = true;
                } else {
                    err = "unsupported distribution datatype " + dt;
                    return false;
                }
            }
            if (!progressed) { err = "distributions could not be resolved"; return false; }
            pending.swap(rest);
        }
    }

    // ---- nuclides (setup.cpp:310-467) ----
    std::vector<std::string> nuc_names;
    if (const XmlNode *nn = doc.child("nuclides")) {
        for (const auto &n : nn->children) {
            if (n.name != "nuclide") continue;
            nuc_names.push_back(n.as_string("name"));
            if (const std::string *zaid = n.attr("ZAID")) {
                const std::string fp = xs_dir + "/" + *zaid + ".txt";
                std::string body;
                if (!read_file(fp, body)) { err = "cannot read " + fp; return false; }
                std::istringstream in(body);
                double A;
                if (!(in >> A)) { err = "failed to read A in " + fp; return false; }
                double c1, c2;
                for (int i = 0; i < 3; ++i)
                    if (!(in >> c1 >> c2)) { err = "failed to read Watt parameters in " + fp; return false; }
                const int64_t off = (int64_t)t.xs_E.size();
                double e, s, c, f, nu, nud;
                while (in >> e >> s >> c >> f >> nu >> nud) {
                    if (f != 0.0) { err = fp + ": fissile data (sigma_f != 0) is outside this path"; return false; }
                    t.xs_E.push_back(e);
                    t.xs_S.push_back(s);
                    t.xs_C.push_back(c + f);        // sigma_a = c + f (setup.cpp:371)
                    t.xs_T.push_back(s + c + f);    // sigma_t = s + c + f (setup.cpp:372)
                }
                const int64_t len = (int64_t)t.xs_E.size() - off;
                if (len < 1) { err = fp + ": no cross-section rows"; return false; }
                t.nuc_kind.push_back(N_TABLE);
                t.nuc_A.push_back(A);
                t.nuc_const.push_back(0.0);
                t.nuc_off.push_back(off);
                t.nuc_len.push_back((int32_t)len);
            } else {
                double cap = 0.0;
                for (const auto &r : n.children) {
                    if (!r.attr("xs")) { err = "unknown XS type in nuclide " + nuc_names.back(); return false; }
                    if (r.name != "capture") { err = "user-defined nuclides support capture only"; return false; }
                    cap = r.as_double("xs");
                }
                t.nuc_kind.push_back(N_CONST);
                t.nuc_A.push_back(n.attr("A") ? n.as_double("A") : (double)3.40282346638528859812e+38F);
                t.nuc_const.push_back(cap);
                t.nuc_off.push_back((int64_t)t.xs_E.size());
                t.nuc_len.push_back(0);
            }
        }
    }

    // ---- materials (setup.cpp:474-492) ----
    std::vector<std::vector<int32_t>> mat_nuc;
    if (const XmlNode *mn = doc.child("materials")) {
        for (const auto &m : mn->children) {
            if (m.name != "material") continue;
            t.mat_names.push_back(m.as_string("name"));
            mat_nuc.emplace_back();
            if (G > 0) {
                const XmlNode *mg = m.child("multigroup");
                if (!mg) { err = "multigroup problem needs <multigroup> data in material " + t.mat_names.back(); return false; }
                const std::vector<double> tot = doubles(mg->as_string("total"));
                const std::vector<double> sca = doubles(mg->as_string("scatter"));
                if ((int)tot.size() != G || (int)sca.size() != G * G) { err = "multigroup data has the wrong size"; return false; }
                t.mg_total.insert(t.mg_total.end(), tot.begin(), tot.end());
                t.mg_scatter.insert(t.mg_scatter.end(), sca.begin(), sca.end());
                for (int g = 0; g < G; ++g) {
                    double acc = 0.0;
                    for (int g2 = 0; g2 < G; ++g2) acc += sca[(size_t)g * G + g2];
                    t.mg_scat_tot.push_back(acc);
                    t.mg_capture.push_back(tot[g] - acc);
                }
                continue;
            }
            for (const auto &n : m.children) {
                if (n.name != "nuclide") continue;
                const int idx = index_of(nuc_names, n.as_string("name"));
                if (idx < 0) { err = "unknown nuclide " + n.as_string("name"); return false; }
                mat_nuc.back().push_back(idx);
                t.mat_dens.push_back(n.as_double("density"));
            }
        }
    }
    {
        std::vector<int32_t> flat;
        offsets_from(mat_nuc, t.mat_off, flat);
        t.mat_nuc = flat;
    }

    // ---- surfaces (setup.cpp:499-584) ----
    if (const XmlNode *sn = doc.child("surfaces")) {
        for (const auto &s : sn->children) {
            const std::string bc = s.as_string("bc", "transmission");
            int32_t bcv;
            if (bc == "transmission") bcv = 0;
            else if (bc == "reflective") bcv = 1;
            else if (bc == "vacuum") bcv = -1;
            else { err = "unknown boundary condition " + bc; return false; }
            double c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            int32_t type;
            if (s.name == "plane_x") { type = S_PX; c[0] = s.as_double("x"); }
            else if (s.name == "plane_y") { type = S_PY; c[0] = s.as_double("y"); }
            else if (s.name == "plane_z") { type = S_PZ; c[0] = s.as_double("z"); }
            else if (s.name == "plane") {
                type = S_PLANE;
                const double a = s.as_double("a"), b = s.as_double("b"), cc = s.as_double("c"), d = s.as_double("d");
                const double L = 2.0 / (a * a + b * b + cc * cc);   // Geometry.cpp:19-22
                c[0] = a; c[1] = b; c[2] = cc; c[3] = d; c[4] = L * a; c[5] = L * b; c[6] = L * cc;
            } else if (s.name == "sphere") {
                type = S_SPHERE;
                const double r = s.as_double("r");
                c[0] = s.as_double("x"); c[1] = s.as_double("y"); c[2] = s.as_double("z"); c[3] = r; c[4] = r * r;
            } else if (s.name == "cylinder_x") {
                type = S_CYLX;
                const double r = s.as_double("r");
                c[0] = s.as_double("y"); c[1] = s.as_double("z"); c[2] = r; c[3] = r * r;
            } else if (s.name == "cylinder_z") {
                type = S_CYLZ;
                const double r = s.as_double("r");
                c[0] = s.as_double("x"); c[1] = s.as_double("y"); c[2] = r; c[3] = r * r;
            } else {
                err = "unknown surface type " + s.name;
                return false;
            }
            t.surf_names.push_back(s.as_string("name"));
            t.surf_type.push_back(type);
            t.surf_bc.push_back(bcv);
            t.surf_coef.insert(t.surf_coef.end(), c, c + 8);
        }
    }

    // ---- cells (setup.cpp:591-629) ----
    std::vector<std::vector<int32_t>> cell_surf;
    if (const XmlNode *cn = doc.child("cells")) {
        for (const auto &c : cn->children) {
            if (c.name != "cell") continue;
            t.cell_names.push_back(c.attr("name") ? c.as_string("name")
                                                  : "Cell " + std::to_string(t.cell_names.size() + 1));
            t.cell_imp.push_back(c.attr("importance") ? c.as_double("importance") : 1.0);
            int32_t mat = -1;
            if (c.attr("material")) {
                mat = index_of(t.mat_names, c.as_string("material"));
                if (mat < 0) { err = "unknown material in cell " + t.cell_names.back(); return false; }
            }
            t.cell_mat.push_back(mat);
            cell_surf.emplace_back();
            for (const auto &s : c.children) {
                if (s.name != "surface") continue;
                const int si = index_of(t.surf_names, s.as_string("name"));
                if (si < 0) { err = "unknown surface " + s.as_string("name"); return false; }
                cell_surf.back().push_back(si);
                t.cell_sense.push_back((int32_t)s.as_int("sense"));
            }
        }
    }
    offsets_from(cell_surf, t.cell_surf_off, t.cell_surf);

    // ---- estimators (setup.cpp:637-805) ----
    std::vector<std::vector<int32_t>> cell_tl(t.cell_imp.size()), cell_c(t.cell_imp.size()),
        surf_est(t.surf_type.size());
    t.est_score_off.assign(1, 0);
    t.est_filt_off.assign(1, 0);
    t.est_factor_off.assign(1, 0);
    t.est_bin_off.assign(1, 0);
    if (const XmlNode *en = doc.child("estimators")) {
        for (const auto &e : en->children) {
            if (e.name != "estimator") continue;
            const int ei = (int)t.est_names.size();
            t.est_names.push_back(e.attr("name") ? e.as_string("name") : "Estimator #" + std::to_string(ei + 1));
            const std::string etype = e.as_string("type", "TL");
            int32_t kernel;
            if (etype == "TL") kernel = K_TL;
            else if (etype == "C") kernel = K_C;
            else { err = "unsupported estimator type in " + t.est_names.back(); return false; }
            if (!e.attr("scores")) { err = "no score in estimator " + t.est_names.back(); return false; }
            std::istringstream iss(e.as_string("scores"));
            t.est_score_names.emplace_back();
            int nscores = 0;
            for (std::string sname; iss >> sname;) {
                int32_t kind;
                if (sname == "flux") kind = SC_FLUX;
                else if (sname == "absorption") kind = SC_ABSORPTION;
                else if (sname == "scatter") kind = SC_SCATTER;
                else if (sname == "capture") kind = SC_CAPTURE;
                else if (sname == "total") kind = SC_TOTAL;
                else if (sname == "cross") { kernel = K_NEUTRON; kind = SC_FLUX; }  // setup.cpp:688-690
                else { err = "unsupported score " + sname + " in estimator " + t.est_names.back(); return false; }
                t.score_kind.push_back(kind);
                t.score_kernel.push_back(kernel);
                t.est_score_names.back().push_back(sname);
                ++nscores;
            }
            t.est_score_off.push_back((int32_t)t.score_kind.size());
            struct Filt { int32_t kind; std::vector<double> grid; int32_t size; };
            std::vector<Filt> filters;
            std::vector<double> grid;
            bool has_surf = false, has_cell = false;
            for (const auto &c : e.children) {
                if (c.name == "surface") {
                    const int si = index_of(t.surf_names, c.as_string("name"));
                    if (si < 0) { err = "unknown surface " + c.as_string("name") + " in estimator " + t.est_names.back(); return false; }
                    surf_est[si].push_back(ei);
                    grid.push_back((double)si);
                    has_surf = true;
                }
            }
            for (const auto &c : e.children) {
                if (c.name == "cell") {
                    const int ci = index_of(t.cell_names, c.as_string("name"));
                    if (ci < 0) { err = "unknown cell " + c.as_string("name") + " in estimator " + t.est_names.back(); return false; }
                    if (etype == "TL") cell_tl[ci].push_back(ei);
                    else cell_c[ci].push_back(ei);
                    grid.push_back((double)ci);
                    has_cell = true;
                }
            }
            if (has_surf && has_cell) { err = "estimator " + t.est_names.back() + " is attached to surfaces and cells"; return false; }
            if (has_surf) filters.push_back({F_SURFACE, grid, (int32_t)grid.size()});
            else if (has_cell) filters.push_back({F_CELL, grid, (int32_t)grid.size()});
            else { err = "estimator " + t.est_names.back() + " needs to be attached somewhere"; return false; }
            for (const auto &f : e.children) {
                if (f.name != "filter") continue;
                const std::string ft = f.as_string("type");
                if (ft == "group") {
                    if (G <= 0) { err = "group filter needs a multigroup problem"; return false; }
                    std::vector<double> g;
                    for (int k = 0; k <= G; ++k) g.push_back((double)k);
                    filters.push_back({F_GROUP, g, G});
                    continue;
                }
                std::vector<double> fg;
                if (f.attr("grid")) {
                    fg = doubles(f.as_string("grid"));
                } else if (f.attr("grid_linear")) {
                    std::vector<double> v = doubles(f.as_string("grid_linear"));
                    v.resize(3, 0.0);
                    const double a = v[0], step = v[1], b = v[2];
                    fg.push_back(a);
                    while (fg.back() < b) fg.push_back(fg.back() + step);
                    fg.pop_back();
                    fg.push_back(b);
                } else if (f.attr("grid_lethargy")) {
                    std::vector<double> v = doubles(f.as_string("grid_lethargy"));
                    v.resize(3, 0.0);
                    const double a = v[0], b = v[1], N = v[2];
                    const double step = plog(b / a) / N;
                    fg.push_back(0.0);
                    while ((double)fg.size() != N + 1) fg.push_back(fg.back() + step);
                    for (size_t i = 0, j = fg.size() - 1; i < j; ++i, --j) std::swap(fg[i], fg[j]);
                    for (double &x : fg) x = b * pexp(-x);
                } else {
                    err = "need filter grid for estimator " + t.est_names.back();
                    return false;
                }
                if (fg.size() < 2) { err = "filter grid needs two points"; return false; }
                if (ft == "energy") filters.push_back({F_ENERGY, fg, (int32_t)fg.size() - 1});
                else if (ft == "time") filters.push_back({F_TIME, fg, (int32_t)fg.size() - 1});
                else { err = "unknown filter type for estimator " + t.est_names.back(); return false; }
            }
            if (filters.size() > 8) { err = "at most 8 filters per estimator"; return false; }
            int64_t ntally = nscores;
            for (const auto &f : filters) {
                t.filt_kind.push_back(f.kind);
                t.filt_size.push_back(f.size);
                t.filt_grid_off.push_back((int64_t)t.filt_grid.size());
                t.filt_grid_len.push_back((int32_t)f.grid.size());
                t.filt_grid.insert(t.filt_grid.end(), f.grid.begin(), f.grid.end());
                ntally *= f.size;
            }
            t.est_filt_off.push_back((int32_t)t.filt_kind.size());
            // Estimator::initialize_tallies (Estimator.cpp:280-295)
            std::vector<double> fac(1, 1.0);
            double factor = 1.0;
            for (int i = (int)filters.size() - 1; i >= 0; --i) {
                factor *= filters[i].size;
                fac.insert(fac.begin(), factor);
            }
            t.est_factor.insert(t.est_factor.end(), fac.begin(), fac.end());
            t.est_factor_off.push_back((int32_t)t.est_factor.size());
            t.est_bin_off.push_back(t.est_bin_off.back() + ntally);
        }
    }
    offsets_from(cell_tl, t.cell_tl_off, t.cell_tl);
    offsets_from(cell_c, t.cell_c_off, t.cell_c);
    offsets_from(surf_est, t.surf_est_off, t.surf_est);

    // ---- sources (setup.cpp:1020-1066) ----
    if (const XmlNode *srcn = doc.child("sources")) {
        for (const auto &s : srcn->children) {
            PointDist dir{};
            dir.kind = D_ISO;
            ScalarDist en{E_DELTA, 2e6, 0.0};
            if (s.attr("direction")) {
                auto it = pdist.find(s.as_string("direction"));
                if (it == pdist.end()) { err = "unknown direction distribution in source"; return false; }
                dir = it->second;
            }
            if (s.attr("energy")) {
                auto it = ddist.find(s.as_string("energy"));
                if (it == ddist.end()) { err = "unknown energy distribution in source"; return false; }
                en = it->second;
            }
            if (s.name != "point") { err = "unknown source type: " + s.name; return false; }
            const double p[3] = {s.as_double("x"), s.as_double("y"), s.as_double("z")};
            int cell = -1;
            for (int c = 0; c < t.n_cell() && cell < 0; ++c) {   // search_cell, general.cpp:26-34
                bool in = true;
                for (int i = t.cell_surf_off[c]; i < t.cell_surf_off[c + 1]; ++i)
                    if (surface_eval_host(t, t.cell_surf[i], p) * t.cell_sense[i] < 0) { in = false; break; }
                if (in) cell = c;
            }
            if (cell < 0) { err = "source point lies in no cell"; return false; }
            const int g = (int)s.as_int("group", 0);
            if (G > 0 && (g < 0 || g >= G)) { err = "source group out of range"; return false; }
            t.src_pos.insert(t.src_pos.end(), p, p + 3);
            t.src_cell.push_back(cell);
            t.src_dir_kind.push_back(dir.kind);
            t.src_dir_par.insert(t.src_dir_par.end(), dir.par, dir.par + 9);
            t.src_e_kind.push_back(en.kind);
            t.src_e_par.push_back(en.a);
            t.src_e_par.push_back(en.range);
            t.src_group.push_back(g);
        }
    }
    if (t.src_cell.empty()) { err = "no source"; return false; }
    // SourceBank::set_up (Source.cpp:65-72): equal steps, probabilities ignored
    t.src_cdf.assign(t.src_cell.size() + 1, 0.0);
    const double dp = 1.0 / (double)t.src_cell.size();
    for (size_t i = 1; i < t.src_cdf.size(); ++i) t.src_cdf[i] = t.src_cdf[i - 1] + dp;
    if (G == 0) {
        for (int m = 0; m < t.n_mat(); ++m)
            if (t.mat_off[m + 1] == t.mat_off[m]) { err = "material " + t.mat_names[m] + " has no nuclide"; return false; }
    }
    return true;
}

}  // namespace mc
