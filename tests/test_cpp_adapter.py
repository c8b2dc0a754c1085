"""include/mcgpu_simulator.hpp: the reference's Simulator interface over the
C ABI.  A program written the way the reference's own integral test is
(test/test_integral_Simulator.cpp:12-27) compiles as C++11 against it
(CPU), and on the GPU reproduces the purely absorbing slab's analytic
leakage."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "mc-old_gb300", "mcgpu")

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include "mcgpu_simulator.hpp"

int main(int argc, char **argv)
{
    mcgpu::Simulator Sim(std::string(argv[1]) + "/", std::string(argv[1]) + "/xs_library");
    Sim.mode = MC_FP64_REPLAY;
    Sim.start();
    const double mean = Sim.Estimators[0]->tally(0).mean;
    const double uncer = Sim.Estimators[0]->tally(0).uncer;
    std::printf("%.17g %.17g %llu %llu %s\n", mean, uncer, Sim.Nsample, Sim.Ntrack,
                Sim.Estimators[0]->name().c_str());
    Sim.report(std::string(argv[1]) + "/");
    return 0;
}
'''


def _compile(tmp, link):
    src = os.path.join(tmp, "prog.cpp")
    with open(src, "w") as f:
        f.write(PROGRAM)
    exe = os.path.join(tmp, "prog")
    cmd = ["g++", "-std=c++11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src]
    if link:
        cmd += ["-L", LIBDIR, "-lmcgpu", "-Wl,-rpath," + LIBDIR, "-o", exe]
    else:
        cmd += ["-fsyntax-only"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_compiles_as_cxx11():
    with tempfile.TemporaryDirectory() as tmp:
        _compile(tmp, link=False)


@pytest.mark.gpu
def test_adapter_runs_the_reference_integral_case():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "mc-old_gb300"))
    import build as B
    B.build()
    import cases
    with tempfile.TemporaryDirectory() as tmp:
        exe = _compile(tmp, link=True)
        d = os.path.join(tmp, "slab")
        os.makedirs(d)
        cases.absorber_slab_user_nuclides(d, samples=100_000)
        r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        mean, uncer, nsample, ntrack, name = r.stdout.split()
        assert os.path.exists(os.path.join(d, "output.json"))
    mean, uncer = float(mean), float(uncer)
    assert int(nsample) == 100_000 and int(ntrack) > 0
    # the reference's own check is |mean - e^-4.2| <= uncer; three sigma here
    assert abs(mean - 0.0149956) <= 3 * uncer
