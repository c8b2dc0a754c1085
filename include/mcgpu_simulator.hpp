/*
 * mcgpu_simulator.hpp -- MC-old's Simulator interface (include/simulator.h)
 * over the C ABI of mcgpu.h, header only.
 *
 * Code written against the reference keeps compiling and running:
 *
 *     Simulator S(io_dir);                               // setup.cpp:30
 *     S.start();                                         // handler.cpp:11
 *     double m = S.Estimators[i]->tally(j).mean;         // Estimator.cpp:424
 *     double u = S.Estimators[i]->tally(j).uncer;
 *     S.report(io_dir);                                  // report.cpp:9
 *
 * Differences: failures throw std::runtime_error with the library's message
 * (the reference exits); report() writes io_dir + "output.json" (the
 * output.h5 tree as JSON); the mode, seed and cross-section directory can be
 * set before start() (the reference has one fixed-source mode, its LCG and
 * ./xs_library).
 */
#ifndef MCGPU_SIMULATOR_HPP
#define MCGPU_SIMULATOR_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mcgpu.h"

namespace mcgpu {

/* Estimator.h:257-270: one tally bin's statistics */
struct Tally {
    double mean = 0.0, uncer = 0.0;
};

inline void check(mc_status s, const mc_problem *p, const char *what)
{
    if (s != MC_OK)
        throw std::runtime_error(std::string(what) + ": " + mc_status_string(s) + ": " + (p ? mc_last_error(p) : ""));
}

/* Estimator: tally(i) and tally_size() (Estimator.cpp:424-432) */
class Estimator {
public:
    Estimator(mc_problem *p, uint32_t e) : p_(p), e_(e)
    {
        char buf[256];
        if (mc_estimator_name(p_, e_, buf, sizeof buf) == MC_OK) name_ = buf;
    }
    unsigned long long tally_size() const
    {
        uint64_t n = 0;
        check(mc_tally_size(p_, e_, &n), p_, "tally_size");
        return n;
    }
    Tally tally(int i) const
    {
        const uint64_t n = tally_size();
        if (i < 0 || (uint64_t)i >= n) throw std::out_of_range("tally index");
        std::vector<double> m(n), s(n);
        check(mc_tally_read(p_, e_, m.data(), s.data(), nullptr, nullptr, n), p_, "tally");
        Tally t;
        t.mean = m[i];
        t.uncer = s[i];
        return t;
    }
    const std::string &name() const { return name_; }

private:
    mc_problem *p_;
    uint32_t e_;
    std::string name_;
};

class Simulator {
public:
    unsigned long long Nsample = 0;   // simulator.h: histories per cycle
    unsigned long long Ntrack = 0;    // simulator.h:109: flights so far
    std::vector<std::shared_ptr<Estimator>> Estimators;

    mc_mode mode = MC_MIXED_EVENT;
    uint64_t seed = 0x4D43;

    explicit Simulator(const std::string io_dir, const std::string xs_dir = "./xs_library")
    {
        mc_problem *p = nullptr;
        const mc_status s = mc_problem_load_xml(io_dir.c_str(), xs_dir.c_str(), &p);
        if (s != MC_OK) {
            const std::string msg = std::string("setup: ") + mc_status_string(s) + ": " + (p ? mc_last_error(p) : "");
            if (p) mc_problem_free(p);
            throw std::runtime_error(msg);
        }
        p_ = p;
        uint64_t n = 0;
        mc_nsample(p_, &n);
        Nsample = n;
        uint32_t ne = 0;
        mc_tally_count(p_, &ne);
        for (uint32_t e = 0; e < ne; ++e) Estimators.push_back(std::make_shared<Estimator>(p_, e));
    }
    Simulator(const Simulator &) = delete;
    Simulator &operator=(const Simulator &) = delete;
    ~Simulator() { mc_problem_free(p_); }

    /* handler.cpp:11-48: Nsample histories (one active cycle) */
    void start()
    {
        check(mc_run(p_, 0, Nsample, seed, mode, nullptr), p_, "start");
        mc_counters c;
        mc_counters_read(p_, &c);
        Ntrack += c.flights;
    }

    /* report.cpp:9-50, as io_dir + "output.json" */
    void report(const std::string io_dir) const
    {
        check(mc_report(p_, (io_dir + "output.json").c_str()), p_, "report");
    }

    mc_problem *handle() const { return p_; }

private:
    mc_problem *p_ = nullptr;
};

}  // namespace mcgpu

#endif
