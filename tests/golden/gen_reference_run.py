"""Generate a large-sample fixture of the compiled reference on the
benchmark workload (the continuous-energy three-shell shield with
20,000-point tables).

Runs oracle/_ref/mcref (the reference's own objects with the test shim, built
by oracle/ref/Makefile) in K processes with K different Philox seeds, each on
histories [0, N) of the workload, and combines the K independent estimates:
per bin, the mean of the K means and the standard error sqrt(sum sigma_k^2)/K.
Writes tests/golden/ce_sphere_bench_run.json with the means, uncertainties,
seeds and history counts.  The production-mode tests compare the GPU's
mixed-precision tallies with it bin by bin (combined 3 sigma, chi-square).
Needs the reference sources, so it runs in the build container only; the
fixture is committed.

    python tests/golden/gen_reference_run.py --ref /path/to/MC-old [--procs 16] [--per-proc 1250000]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases  # noqa: E402
import gen_golden  # noqa: E402

SEED0 = 0x4D43 + 0x10000


def parse(out: str):
    est = []
    for line in out.split("\n"):
        p = line.split()
        if not p or p[0] in ("Ntrack", "Nsample", "estimators"):
            continue
        if p[0] == "estimator":
            est.append([])
        else:
            est[-1].append((float.fromhex(p[0]), float.fromhex(p[1])))
    return est


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MC_OLD_REF"),
                    help="path of the MC-old checkout (default: $MC_OLD_REF)")
    ap.add_argument("--procs", type=int, default=16)
    ap.add_argument("--per-proc", type=int, default=1_250_000)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set MC_OLD_REF to the MC-old checkout")
    gen_golden.build_reference(a.ref)
    with tempfile.TemporaryDirectory() as d:
        cases.ce_sphere_bench(d, samples=a.per_proc)
        seeds = [SEED0 + k for k in range(a.procs)]

        def one(seed):
            r = subprocess.run([gen_golden.MCREF, d, str(seed)], cwd=d, capture_output=True, text=True,
                               check=True)
            return parse(r.stdout)

        t0 = time.perf_counter()
        with ThreadPoolExecutor(a.procs) as ex:
            runs = list(ex.map(one, seeds))
        wall = time.perf_counter() - t0
    K = len(runs)
    out = {"case": "ce_sphere_bench", "generator": "tests/golden/gen_reference_run.py (compiled reference + oracle/ref shim)",
           "seeds": seeds, "histories_per_seed": a.per_proc, "histories": K * a.per_proc,
           "combine": "mean of the per-seed means; sqrt(sum of squared standard errors) / K",
           "estimators": []}
    for e in range(len(runs[0])):
        m = np.array([[b[0] for b in r[e]] for r in runs])
        s = np.array([[b[1] for b in r[e]] for r in runs])
        mean = m.mean(axis=0)
        unc = np.sqrt((s ** 2).sum(axis=0)) / K
        out["estimators"].append([[float(x).hex(), float(y).hex()] for x, y in zip(mean, unc)])
    with open(os.path.join(HERE, "ce_sphere_bench_run.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"{K} x {a.per_proc} histories in {wall:.1f} s wall")


if __name__ == "__main__":
    main()
