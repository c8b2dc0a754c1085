"""Generate the golden fixtures from the compiled reference.

Runs the reference's own objects (built from the MC-old sources by
oracle/ref/Makefile into oracle/_ref/mcref) on every case of cases.py and
writes tests/golden/<case>.json: Ntrack, each estimator's tally mean and
uncertainty as C99 hex floats, and a SHA-256 of the per-history event
digests.  Needs the reference sources, so it runs in the build container
only; the fixtures it writes are committed and travel everywhere.

    python tests/golden/gen_golden.py --ref /path/to/MC-old   (or MC_OLD_REF=...)
"""
import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
import cases  # noqa: E402

MCREF = os.path.join(ROOT, "oracle", "_ref", "mcref")


def build_reference(ref: str) -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}", "-j8"],
                   check=True)


def run_reference(case_dir: str, seed: int):
    dig = os.path.join(case_dir, "digest.bin")
    out = subprocess.run([MCREF, case_dir, str(seed), "--digest", dig], cwd=case_dir,
                         capture_output=True, text=True, check=True).stdout.split("\n")
    res = {"ntrack": 0, "estimators": []}
    for line in out:
        p = line.split()
        if not p:
            continue
        if p[0] == "Ntrack":
            res["ntrack"] = int(p[1])
        elif p[0] == "Nsample":
            res["nsample"] = int(p[1])
        elif p[0] == "estimator":
            res["estimators"].append([])
        elif p[0] not in ("estimators",):
            res["estimators"][-1].append([p[0], p[1]])
    d = np.fromfile(dig, dtype=np.uint64)
    res["digest_sha256"] = hashlib.sha256(d.tobytes()).hexdigest()
    res["digest_head"] = [f"{int(v):016x}" for v in d[:8]]
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MC_OLD_REF"),
                    help="path of the MC-old checkout (default: $MC_OLD_REF)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set MC_OLD_REF to the MC-old checkout")
    build_reference(args.ref)
    for name in cases.REFERENCE_CASES:
        with tempfile.TemporaryDirectory() as d:
            cases.write_case(name, d)
            res = run_reference(d, cases.SEED)
        res.update({"case": name, "seed": cases.SEED,
                    "generator": "tests/golden/gen_golden.py (compiled reference + oracle/ref shim)"})
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(res, f, indent=1)
        print(name, "Ntrack", res["ntrack"], "bins", sum(len(e) for e in res["estimators"]))


if __name__ == "__main__":
    main()
