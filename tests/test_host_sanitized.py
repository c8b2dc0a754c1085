"""The library's host-side readers (input.xml, cross-section tables, the
FP32 table builder) under AddressSanitizer and UndefinedBehaviorSanitizer:
tests/host_parse_check.cpp, linked with mc_xml.cpp, mc_problem.cpp and
mc_evtables.cpp, loads every golden case, the benchmark workloads and every
malformed input of test_abi without a sanitizer report, accepting the good
inputs and refusing the bad ones."""
import os
import shutil
import subprocess
import tempfile

import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mc-old_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def _build(out):
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off",
           "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", CUDA_INC,
           os.path.join(ROOT, "tests", "host_parse_check.cpp"),
           os.path.join(CSRC, "mc_xml.cpp"), os.path.join(CSRC, "mc_problem.cpp"),
           os.path.join(CSRC, "mc_evtables.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("no sanitizer runtime for g++ here")
    assert r.returncode == 0, r.stderr[-3000:]


def test_host_readers_are_clean_under_asan_and_ubsan():
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers are missing")
    import mcgpu.workloads as W
    from test_abi import BAD_INPUTS
    with tempfile.TemporaryDirectory() as root:
        exe = os.path.join(root, "host_parse_check")
        _build(exe)
        good, bad = [], []
        for name in cases.REFERENCE_CASES:
            d = os.path.join(root, "g_" + name)
            cases.write_case(name, d)
            good.append((d, os.path.join(d, "xs_library")))
        for name, writer in (("ce_sphere", lambda d: W.ce_sphere(d, samples=100, n_points=2000)),
                             ("slab_1g", lambda d: W.slab_1g(d, samples=100)),
                             ("mg_deep_slab", lambda d: W.mg_deep_slab(d, samples=100)),
                             ("mg_layered_slab", lambda d: W.mg_layered_slab(d, samples=100))):
            d = os.path.join(root, "w_" + name)
            os.makedirs(d)
            writer(d)
            good.append((d, os.path.join(d, "xs_library")))
        for k, (case, body) in enumerate(BAD_INPUTS.items()):
            d = os.path.join(root, "b%d" % k)
            os.makedirs(d)
            if case == "fission":   # a fissile table, as test_abi writes it
                os.makedirs(os.path.join(d, "xs_library"))
                with open(os.path.join(d, "xs_library", "092235.txt"), "w") as f:
                    f.write("235\n0 0\n0 0\n0 0\n1e-5 10 5 100 2.4 0\n2e7 4 0.1 1 2.6 0\n")
                body = '<nuclides><nuclide name="U" ZAID="092235"/></nuclides>'
            with open(os.path.join(d, "input.xml"), "w") as f:
                f.write("<?xml version='1.0'?>\n" + body + "\n")
            bad.append((d, os.path.join(d, "xs_library")))
        args = [x for pair in good + bad for x in pair]
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1",
                   UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
        r = subprocess.run([exe] + args, capture_output=True, text=True, env=env, timeout=600)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-4000:]
    assert "Sanitizer" not in out and "runtime error" not in out, out[-4000:]
    lines = r.stdout.splitlines()
    assert len(lines) == len(good) + len(bad)
    assert all(l.startswith("ok") for l in lines[:len(good)]), lines[:len(good)]
    assert all(l.startswith("err") for l in lines[len(good):]), lines[len(good):]
