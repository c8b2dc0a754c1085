// shim_sim.cpp -- history loop around the reference's own objects.
//
// Test infrastructure (reference build for the CPU oracle).  Replaces the
// reference's src/simulator/general.cpp, handler.cpp and fixed_source.cpp
// with re-definitions of the same Simulator members (declared, unchanged, in
// the reference's include/simulator.h).  Everything the loop calls --
// Particle, Surface, Cell, Material, Nuclide, XSTable, ReactionScatter,
// Distribution, SourceBank, Estimator, weight_roulette and cell_importance --
// is the reference's compiled code.  The loop itself follows
// general.cpp:13-211 and handler.cpp:11-48 with three changes:
//   1. the implicit-fission block (general.cpp:135-151) is skipped and draws
//      nothing (fission is out of scope; the reference dereferences a null
//      nuclide there in every non-fissile medium, fixed_source.cpp:15);
//   2. the Philox context (history, particle id, event, draw) is advanced
//      once per random-walk iteration, and particles copied by importance
//      splitting get derived ids;
//   3. wr / ws can be overridden, and a per-history event digest is kept;
//   4. when the input asks for the particle comb, the combed bank's copies get
//      fresh particle ids (the comb itself is the reference's particle_comb).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "simulator.h"
#include "Algorithm.h"
#include "Random.h"
#include "shim_rng.h"

// set by shim_main.cpp
bool g_shim_wr_set = false;
double g_shim_wr = 0.001, g_shim_ws = 1.0;
uint64_t g_shim_seed = 0x4D43;
std::vector<uint64_t> g_shim_digest;

static std::vector<uint32_t> s_ids;   // particle ids parallel to Pbank
// the comb's draw and the combed copies' ids use this event number, which no
// random walk reaches
static const uint32_t kCombEvent = 0xFFFFFFFFu;
static uint64_t s_digest;

static inline void dig(uint64_t v) { s_digest = (s_digest ^ v) * 0x100000001B3ULL; }
static inline uint64_t bits(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }

bool Simulator::test_point(const Point &p, const std::shared_ptr<Cell> &C)
{
    for (const auto &S : C->surfaces()) {
        if (S.first->eval(p) * S.second < 0) { return false; }
    }
    return true;
}

std::shared_ptr<Cell> Simulator::search_cell(const Point &p)
{
    for (const auto &C : Cells) {
        if (test_point(p, C)) { return C; }
    }
    std::fprintf(stderr, "[shim] particle lost at (%a, %a, %a)\n", p.x, p.y, p.z);
    std::exit(3);
}

double Simulator::collision_distance(const Particle &P)
{
    if (P.cell()->material()) {
        return exponential_sample(P.cell()->material()->SigmaT(P.energy()));
    }
    return MAX_float_less;
}

std::pair<std::shared_ptr<Surface>, double> Simulator::surface_intersect(const Particle &P)
{
    double dist = MAX_float;
    std::shared_ptr<Surface> S = nullptr;
    for (const auto &s : P.cell()->surfaces()) {
        double d = s.first->distance(P);
        if (d < dist) { dist = d; S = s.first; }
    }
    return std::make_pair(S, dist);
}

void Simulator::move_particle(Particle &P, const double l)
{
    P.move(l);
    Ntrack++;
    if (tally) {
        for (auto &e : P.cell()->estimators_TL) { e->score(P, l); }
    }
}

void Simulator::surface_hit(Particle &P, const std::shared_ptr<Surface> &S)
{
    P.set_surface_old(S);
    if (S->bc() == 0) {
        P.move(EPSILON_float);
        P.set_cell(search_cell(P.pos()));
    } else if (S->bc() == -1) {
        P.kill();
        P.set_cell(P.cell());
    } else {
        S->reflect(P);
        P.move(EPSILON_float);
        P.set_cell(P.cell());
    }
    if (tally) {
        for (auto &e : S->estimators) { e->score(P, 0.0); }
    }
    const size_t before = Pbank.size();
    cell_importance(P, Pbank);
    for (size_t k = before; k < Pbank.size(); ++k) {
        s_ids.push_back(orc_child_id(g_shim_rng.id, g_shim_rng.event, (uint32_t)(k - before + 1)));
    }
}

void Simulator::collision(Particle &P)
{
    if (!P.cell()->material()) { return P.kill(); }
    if (tally) {
        for (auto &e : P.cell()->estimators_C) { e->score(P, 0); }
    }
    std::shared_ptr<Material> M = P.cell()->material();
    // implicit fission skipped: Sigma_f == 0 for every nuclide in scope
    const double implicit = M->SigmaC(P.energy()) + 0.0;
    P.set_weight(P.weight() * (M->SigmaT(P.energy()) - implicit) / M->SigmaT(P.energy()));
    std::shared_ptr<Nuclide> N_scatter = M->nuclide_scatter(P.energy());
    if (!N_scatter) { return; }
    N_scatter->scatter()->sample(P);
}

void Simulator::push_particle_bank(const Particle &P)
{
    Pbank.push_back(P);
    s_ids.push_back(0);
}

static void digest_event(const Particle &P, uint64_t type)
{
    dig(type | ((uint64_t)(uint32_t)P.cell()->ID() << 8));
    const Point x = P.pos(), u = P.dir();
    dig(bits(x.x)); dig(bits(x.y)); dig(bits(x.z));
    dig(bits(u.x)); dig(bits(u.y)); dig(bits(u.z));
    dig(bits(P.energy()));
    dig(bits(P.weight()));
}

void Simulator::random_walk(Particle &P)
{
    g_shim_rng.event = 0;
    dig(0xA5A5A5A5ULL ^ g_shim_rng.id);
    while (P.alive()) {
        g_shim_rng.event++;
        g_shim_rng.draw = 0;
        const std::pair<std::shared_ptr<Surface>, double> SnD = surface_intersect(P);
        double dcol = collision_distance(P);
        uint64_t type;
        if (dcol > SnD.second) {
            move_particle(P, SnD.second);
            surface_hit(P, SnD.first);
            type = 1;
        } else {
            move_particle(P, dcol);
            collision(P);
            type = 2;
        }
        weight_roulette(P);
        digest_event(P, type);
    }
}

void Simulator::start()
{
    if (g_shim_wr_set) { wr = g_shim_wr; ws = g_shim_ws; }
    g_shim_rng.seed = g_shim_seed;
    g_shim_digest.clear();
    for (icycle = 0; icycle < Ncycle; icycle++) {
        if (icycle == Npassive) { tally = true; }
        Sbank = Fbank; Sbank.set_up(); Fbank.reset();
        for (isample = 0; isample < Nsample; isample++) {
            g_shim_rng.history = isample;
            g_shim_rng.id = 0;
            g_shim_rng.event = 0;
            g_shim_rng.draw = 0;
            s_digest = 0xCBF29CE484222325ULL;
            Pbank.push_back(Sbank.get_source());
            s_ids.push_back(0);
            while (!Pbank.empty()) {
                Particle P = Pbank.back(); Pbank.pop_back();
                g_shim_rng.id = s_ids.back(); s_ids.pop_back();
                random_walk(P);
                if (comb) {   // handler.cpp:27, the reference's own particle_comb
                    const uint32_t walker = g_shim_rng.id;
                    const bool acts = Pbank.size() >= (size_t)bank_max;
                    g_shim_rng.event = kCombEvent;
                    g_shim_rng.draw = 0;
                    particle_comb(Pbank);
                    if (acts) {
                        s_ids.resize(Pbank.size());
                        for (size_t k = 0; k < Pbank.size(); ++k)
                            s_ids[k] = orc_child_id(walker, kCombEvent, (uint32_t)(k + 1));
                    }
                }
            }
            if (tally) {
                for (auto &E : Estimators) { E->end_history(); }
            }
            g_shim_digest.push_back(s_digest);
        }
        if (tally) { for (auto &E : Estimators) { E->end_cycle(); } }
    }
    for (auto &E : Estimators) { E->end_simulation(); }
}
