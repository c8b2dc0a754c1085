"""The command-line driver (mcgpu_run, the counterpart of the reference's
MC.exe, Main.cpp:8-31) and the report it writes (the output.h5 tree of
report.cpp:9-50 / Estimator.cpp:368-422, as JSON).  In FP64 replay the
report's means and uncertainties equal the golden values the compiled
reference produced for the same input, bit for bit."""
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

import cases
from helpers import golden_arrays, load_golden, same_bits

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "mc-old_gb300", "mcgpu", "mcgpu_run")


@pytest.fixture(scope="module")
def built():
    import build as B
    B.build()
    return EXE


def _flatten(v):
    return np.asarray(v, dtype=float).reshape(-1)


@pytest.mark.parametrize("name", ["slab_features", "quadrics", "comb_slab"])
def test_driver_report_equals_golden(built, name):
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(name, d)
        r = subprocess.run([built, d, "--mode", "replay", "--xs", os.path.join(d, "xs_library"),
                            "--seed", str(g["seed"])], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Simulation output done!" in r.stdout
        with open(os.path.join(d, "output.json")) as f:
            rep = json.load(f)
    assert rep["summary"]["Ntrack"] == g["ntrack"]
    assert rep["summary"]["Nsample"] == g["nsample"]
    means, uncs = [], []
    for est, val in rep.items():
        if est == "summary":
            continue
        for key, sub in val.items():
            if isinstance(sub, dict) and "mean" in sub:
                means.append(_flatten(sub["mean"]))
                uncs.append(_flatten(sub["uncertainty"]))
    gm, gu = golden_arrays(g)
    assert same_bits(np.concatenate(means), gm) and same_bits(np.concatenate(uncs), gu)


def test_driver_errors_are_exit_codes(built):
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([built, d], capture_output=True, text=True, timeout=120)
        assert r.returncode == 2 + 1, r.stdout + r.stderr    # MC_ERR_INPUT: no input.xml
        assert "[ERROR]" in r.stderr
