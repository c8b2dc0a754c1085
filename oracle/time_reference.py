"""Speed of the compiled reference against the C oracle port on one core.

TEST INFRASTRUCTURE (a timing of the two CPU implementations of the
history loop; the GPU path is not involved).  Both run the benchmark
workload (continuous-energy three-shell shield, 20,000-point tables, 2 MeV
isotropic point source) on the same Philox seed and the same history range
[0, N), one process each, pinned to one core in turn:

  * oracle/_ref/mcref -- the reference's own objects (Particle, Geometry,
    Reaction, Estimator, ... compiled from the MC-old sources by
    oracle/ref/Makefile) with the test shim;
  * the C port (oracle/mc_oracle.c through oracle/problem.py).

mcref's wall time includes reading input.xml and the tables, so its
per-history time is the slope between two history counts; the port is timed
around its history loop alone (and by the same slope, as a check).  Ntrack
of the two must be equal (the port is bit-exact with the reference).
Needs the reference sources (to build mcref), so it runs in the build
container only.

    python oracle/time_reference.py --ref /path/to/MC-old [--n1 4000 --n2 24000 --repeat 3]
"""
import argparse
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, os.path.join(ROOT, "mc-old_gb300")]

MCREF = os.path.join(HERE, "_ref", "mcref")
SEED = 0x4D43 + 1


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def time_mcref(d, n):
    from mcgpu import workloads as W
    W.ce_sphere(d, samples=n)
    t0 = time.perf_counter()
    r = subprocess.run(["taskset", "-c", "0", MCREF, d, str(SEED)], cwd=d, capture_output=True, text=True,
                       check=True)
    wall = time.perf_counter() - t0
    ntrack = int(next(l.split()[1] for l in r.stdout.split("\n") if l.startswith("Ntrack")))
    return wall, ntrack


def time_port(d, n):
    from mcgpu import workloads as W
    from oracle import problem as OP
    W.ce_sphere(d, samples=n)
    t0 = time.perf_counter()
    pb = OP.load(d, xs_dir=os.path.join(d, "xs_library"))
    t1 = time.perf_counter()
    r = OP.run(pb, n=n, seed=SEED)
    t2 = time.perf_counter()
    return t2 - t0, t2 - t1, int(r.counters[0])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MC_OLD_REF"),
                    help="path of the MC-old checkout (default: $MC_OLD_REF)")
    ap.add_argument("--n1", type=int, default=4000)
    ap.add_argument("--n2", type=int, default=24000)
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set MC_OLD_REF to the MC-old checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={a.ref}", "-j8"], check=True)
    subprocess.run(["make", "-s", "-C", HERE, "lib"], check=True)
    os.sched_setaffinity(0, {0})
    best = {}
    with tempfile.TemporaryDirectory() as tmp:
        for n in (a.n1, a.n2):
            for k in range(a.repeat):
                d = os.path.join(tmp, f"ref{n}_{k}")
                w, nt_ref = time_mcref(d, n)
                d = os.path.join(tmp, f"port{n}_{k}")
                wp, loop, nt_port = time_port(d, n)
                assert nt_ref == nt_port, (n, nt_ref, nt_port)
                key = (n,)
                b = best.get(key, (1e30, 1e30, 1e30, nt_ref))
                best[key] = (min(b[0], w), min(b[1], wp), min(b[2], loop), nt_ref)
    (r1, p1, l1, t1), (r2, p2, l2, t2) = best[(a.n1,)], best[(a.n2,)]
    dn = a.n2 - a.n1
    ref_rate = dn / (r2 - r1)
    port_rate = dn / (p2 - p1)
    port_loop = a.n2 / l2
    print(f"cpu: {_cpu_model()}, 1 core; workload ce_sphere (20,000-point tables), seed {SEED:#x}")
    print(f"Ntrack at {a.n1} / {a.n2} histories: {t1} / {t2} (reference = port)")
    print(f"reference (compiled MC-old objects + shim): {ref_rate:,.0f} histories/s (slope, best of {a.repeat})")
    print(f"C oracle port:                               {port_rate:,.0f} histories/s (slope), "
          f"{port_loop:,.0f} histories/s (history loop alone)")
    print(f"port / reference speed: {port_rate / ref_rate:.3f}")


if __name__ == "__main__":
    main()
