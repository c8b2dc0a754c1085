"""bench.py's reference arm runs the C restatement of the reference's history
loop on the host cores (no GPU) and prints one JSON line of the bench
contract with impl = "reference"."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-histories-per-proc", "40"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["unit"] == "histories/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert "ce_sphere" in line["config"]["workload"]


def test_issue_roofline_arithmetic():
    """roofline_issue = committed warp instructions per history x histories/s
    over 4 schedulers per SM x SM clock; absent for shapes without a capture."""
    sys.path.insert(0, ROOT)
    import bench
    prof = {"issue:k_track:6": 6000.0, "slab_1g/issue:k_track:8": 100.0}
    leg = bench.LEGS["ce_sphere"]
    r = bench._issue_roofline(prof, leg, {"kernel": 2, "blocks_per_sm": 6}, 1e8, {"sm_mhz": 2000.0}, 150)
    assert r["bound"] == "issue" and abs(r["peak"] - 150 * 4 * 2e9) < 1
    assert abs(r["achieved"] - 6e11) < 1 and abs(r["frac"] - 0.5) < 1e-12
    assert bench._issue_roofline(prof, leg, {"kernel": 2, "blocks_per_sm": 8}, 1e8, {"sm_mhz": 2000.0}, 150) is None
    assert bench._issue_roofline(prof, leg, {"kernel": 1, "blocks_per_sm": 2}, 1e8, {"sm_mhz": 2000.0}, 150) is None
    r = bench._issue_roofline(prof, bench.LEGS["slab_1g"], {"kernel": 2, "blocks_per_sm": 8}, 1e9,
                              {"sm_mhz": 2000.0}, 150)
    assert abs(r["achieved"] - 1e11) < 1


def test_algorithmic_bytes_per_workload():
    """Continuous energy: 16 B per nuclide lookup and per tally update;
    multigroup: 4 B per cross-section value, 4 B per scatter-CDF probe
    (ceil(log2 G) per collision), 16 B per tally update."""
    sys.path.insert(0, ROOT)
    import bench
    cnt = {"nuc_lookups": 10, "tally_updates": 3, "xs_evals": 7, "collisions": 2}
    assert bench._alg_bytes(bench.LEGS["ce_sphere"], cnt) == 16 * 10 + 16 * 3
    assert bench._alg_bytes(bench.LEGS["mg_deep_slab"], cnt) == 4 * 7 + 4 * 5 * 2 + 16 * 3
    assert bench._alg_bytes(bench.LEGS["mg_layered_slab"], cnt) == 4 * 7 + 16 * 3


def test_reference_arm_runs_every_single_problem_workload():
    for w in ("slab_1g", "mg_deep_slab", "mg_layered_slab"):
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                            "--warmup", "0", "--ref-histories-per-proc", "50", "--workload", w],
                           capture_output=True, text=True, timeout=600, cwd=ROOT)
        assert r.returncode == 0, r.stdout + r.stderr
        line = json.loads([l for l in r.stdout.splitlines() if l.strip().startswith("{")][0])
        assert line["impl"] == "reference" and line["value"] > 0 and w in line["config"]["workload"]


def test_reference_arm_runs_the_batch():
    """The batch on the host cores: one oracle process per core over a
    seeded random sample of its problems."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-seconds", "0.2", "--workload", "batch", "--batch-problems", "16"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    line = json.loads([l for l in r.stdout.splitlines() if l.strip().startswith("{")][0])
    assert line["impl"] == "reference" and line["value"] > 0 and "batch_shields: 16" in line["config"]["workload"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["value"] == line["value"]


def test_batch_cpu_estimate_arithmetic(monkeypatch):
    """The batch's CPU time = its histories x the sampled problems' mean CPU
    time per history, spread over the cores: with every sampled problem at
    a known time per history the rate is cores / mean."""
    sys.path.insert(0, ROOT)
    import bench
    per = {"a": 1e-6, "b": 3e-6, "c": 2e-6, "d": 2e-6}
    monkeypatch.setattr(bench, "_oracle_worker", lambda job: (per[job[0]] * job[2], 0))
    import oracle.problem as OP
    monkeypatch.setattr(OP, "build", lambda: None)
    specs = [("a", 100), ("b", 10_000_000), ("c", 5000), ("d", 70)]
    rate, sampled, ran = bench.cpu_batch_sample(specs, 1e9, procs=1, cap=1000)
    assert sampled == 4 and ran == 100 + 1000 + 1000 + 70
    assert abs(rate - 1.0 / 2e-6) < 1e-6 * rate
