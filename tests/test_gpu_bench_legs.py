"""Every bench.py leg runs and prints one contract line (small sizes): the
metric, the device-timed value, the roofline against the measured HBM peak,
the end-to-end figure through the C ABI, the one-core CPU baseline (for the
batch: a sample of its problems) and, for the single-problem legs, the FOM
and the plain FP64 comparison."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

LEGS = [
    ("ce_sphere", ["--histories", "100000"]),
    ("slab_1g", ["--histories", "100000"]),
    ("mg_deep_slab", ["--histories", "1000000"]),
    ("mg_layered_slab", ["--histories", "1000000"]),
    ("batch", ["--batch-problems", "16"]),
]


@pytest.mark.parametrize("workload,extra", LEGS, ids=[w for w, _ in LEGS])
def test_bench_leg_prints_a_contract_line(workload, extra):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", workload, "--steps", "1",
           "--warmup", "3", "--kernel", "thread", "--e2e-steps", "1", "--cpu-seconds", "0.3",
           "--plain-max-histories", "50000"] + extra
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    line = json.loads(lines[0])
    assert line["unit"] == "histories/s" and line["value"] > 0 and line["n_gpus"] == 1
    assert line["roofline"]["bound"] == "hbm" and line["roofline"]["achieved"] > 0
    assert line["e2e"]["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] > 0
    assert line["gpu_launches"] >= 1 and line["clocks"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] > 0
    if workload != "batch":
        assert line["fom"]["value"] > 0 and 0 < line["fom"]["R"] < 1
        assert line["plain_fp64"]["value"] > 0 and line["plain_fp64"]["fom"] > 0
