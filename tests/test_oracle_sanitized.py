"""Host-side memory and undefined-behaviour check of the CPU oracle: the
oracle built with AddressSanitizer and UndefinedBehaviorSanitizer
(`make -C oracle sanitized`) runs every golden case in a child process with
libasan preloaded, stops at the first report, and still reproduces the
compiled reference's golden tallies bit for bit.  (compute-sanitizer is not
available for the device code; its bounds are checked in the kernels and
reported as status codes.)"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, tempfile
sys.path.insert(0, ROOT); sys.path.insert(0, os.path.join(ROOT, "tests")); sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import numpy as np
import cases
from helpers import golden_arrays, load_golden, same_bits
from oracle import problem as OP
for name in cases.REFERENCE_CASES:
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(name, d)
        r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), seed=g["seed"], n=min(g["nsample"], 400))
    assert r.status == 0, name
    if g["nsample"] <= 400:
        m, s = r.finalize()
        gm, gu = golden_arrays(g)
        assert same_bits(m, gm) and same_bits(s, gu), name
    print("ok", name, flush=True)
"""


def _gcc_lib(name):
    try:
        p = subprocess.run(["gcc", "-print-file-name=" + name], capture_output=True, text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_oracle_is_clean_under_asan_and_ubsan():
    asan = _gcc_lib("libasan.so")
    if asan is None:
        pytest.skip("gcc has no AddressSanitizer runtime here")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "sanitized"], check=True)
    env = dict(os.environ)
    env.update({"LD_PRELOAD": asan, "ASAN_OPTIONS": "detect_leaks=0:abort_on_error=0:halt_on_error=1",
                "UBSAN_OPTIONS": "halt_on_error=1:print_stacktrace=1",
                "MC_ORACLE_LIB": os.path.join(ROOT, "oracle", "_build", "liboracle_san.so")})
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + CHILD], capture_output=True, text=True,
                       env=env, timeout=900, cwd=ROOT)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-4000:]
    assert "AddressSanitizer" not in out and "runtime error" not in out, out[-4000:]
    import cases
    assert out.count("ok ") == len(cases.REFERENCE_CASES), out[-2000:]
