"""Benchmark of the fixed-source particle-history path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode event|plain|replay]
                    [--workload ce_sphere|slab_1g|mg_deep_slab|mg_layered_slab|batch]
                    [--histories H] [--impl reference]

Workloads (the configurations of the benchmark, each at its own size; inputs
are synthetic, numpy PCG64 seeded, see mcgpu/workloads.py):

  ce_sphere        (default) continuous-energy three-shell spherical shield:
                   water-like H1/O16 0-30 cm, graphite 30-60 cm, borated
                   graphite 60-70 cm; 20,000-point log-uniform tables for five
                   nuclides; isotropic 2 MeV point source; leakage current,
                   50-bin lethargy spectrum in the outer shell, per-shell
                   flux; 10^7 histories per step.  The tables (0.8 MB FP32 /
                   1.6 MB FP64) are L2-resident by design.
  slab_1g          1-group 20 cm slab, sigma_t = 1, c = 0.5, inward plane
                   source, 100-bin flux; 10^6 histories per step.
  mg_deep_slab     30-group 100 cm deep-penetration slab, importance 2^r,
                   weight roulette 0.25 -> 1; 10^8 histories per step.
  mg_layered_slab  16-layer one-group slab (sigma_t ~ U[0.5, 2]); 10^7
                   histories per step; the reflected current beside the
                   transmitted one (~5e-9, unresolved at this size).
  batch            4096 uneven multigroup shields in one graph launch.

One step = one mc_run over H histories on a fresh history range.  L2 is
flushed between timed steps with a 256 MiB write.

value      histories/s over all ranks, device time (CUDA events on the
           library's stream) summed over the K timed steps, max over ranks.
fom        1/(R^2 T) of the workload's FOM tally (a tally that reaches
           R <= 1 % in one step; R its relative error after the step, T the
           step's device time), with R; the same for every other tally
           named in fom.tallies.
plain_fp64 the plain FP64 GPU history path (MC_FP64_PLAIN) on the same
           workload after the timed region, run until the FOM tally also
           reaches R <= 1 %: histories/s, R, FOM and the mixed / plain FOM
           ratio at matched R <= 1 %.
e2e        the same metric through the C ABI from the host: per step, the
           problem tables re-uploaded from pinned host memory
           (mc_problem_upload), mc_run, and every tally read back to host
           buffers (mc_tally_read); wall clock.
roofline   the transport kernel against HBM: algorithmic bytes per run from
           the device counters (continuous energy: 16 B x nuclide lookups at
           flights + 16 B x tally bin updates; multigroup: 4 B per
           cross-section value + 4 B per scatter-CDF probe + 16 B per tally
           update), over the kernel's CUDA-event time; peak =
           MEASURED_PEAKS.json hbm_gbs; traffic from the committed ncu
           summary of that workload and launch shape.
roofline_l2  the same algorithmic bytes against an L2 read bandwidth measured
           in the run (the tables are L2-resident).
roofline_issue  the kernel against its issue bound: warp instructions per
           history from the committed ncu capture of the same workload and
           launch shape x histories/s, over 4 schedulers per SM x the sampled
           SM clock (the bound these latency-bound kernels actually have),
           with the capture's warp execution efficiency (active threads per
           warp instruction / 32).
cpu_baseline  the CPU oracle (a C restatement of the reference's history
           loop) on one host core, on a bounded sample (~10 s) of the same
           workload.
merged     (N > 1) every rank's tally sums gathered and merged in rank order
           (mcgpu/parallel.py): the FOM tally over all N x H histories of
           the last step, against rank 0's own estimate.

--impl reference times that CPU implementation (all host threads) as the
reference arm and prints its own JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mc-old_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "histories/s and FOM=1/(σ²T) on 1 GB300, mixed/batched vs plain FP64, vs host CPU"
WORKLOAD = "ce_sphere: CE 3-shell spherical shield, 5 nuclides x 20000-point tables, 2 MeV point source"
SEED = 0x4D43 + 1


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        mhz, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(mhz) if mhz else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(mhz)}


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0}, "fallback"


def _l2_read_gbs(torch):
    """L2 read bandwidth, measured here: one reduction kernel sums each of 64
    rows that all alias the same 32 MiB FP32 buffer (a stride-0 view; the
    buffer stays resident in the 129 MB L2), 2 GiB of reads per launch, over
    the CUDA-event time, best of 5 after warm-up.  MEASURED_PEAKS.json holds
    no L2 figure; the cross-section tables of these workloads live in L2, so
    the algorithmic bytes are also set against this."""
    n, reps = 8 << 20, 64
    a = torch.ones(n, dtype=torch.float32, device="cuda")
    v = a.expand(reps, n)
    out = torch.empty(reps, dtype=torch.float32, device="cuda")
    for _ in range(3):
        torch.sum(v, dim=1, out=out)
    best = 0.0
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.sum(v, dim=1, out=out)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 4.0 * n * reps / (e0.elapsed_time(e1) * 1e-3) / 1e9)
    del a, v, out
    return best


def _shape(tuned):
    """The autotuned launch shape: kernel 1 = particle tile with event queues
    (tile particles per CTA), kernel 2 = one particle per thread, kernel 3 =
    event kernels over the particle bank in HBM."""
    if not tuned:
        return None
    if tuned.get("kernel") == 2:
        return {"kernel": "per-thread (k_track)", "blocks_per_sm": tuned["blocks_per_sm"],
                "refill": tuned.get("refill") or "default"}
    if tuned.get("kernel") == 3:
        return {"kernel": "event kernels over an HBM bank (k_ev_*)", "bank": tuned.get("bank_capacity")}
    return {"kernel": "tile (k_event)", "tile": tuned["bank_capacity"], "blocks_per_sm": tuned["blocks_per_sm"]}


# Each workload: what it is, its histories per step, the writer, the tally
# the FOM is quoted on (estimator name, bin, description: a tally that
# reaches R <= 1 % in one step of either mode), more tallies whose FOM is
# reported beside it, the groups of a multigroup problem (0: continuous
# energy) and the profile key prefix of its committed ncu figures.
LEGS = {
    "ce_sphere": {
        "desc": WORKLOAD, "histories": 10_000_000,
        "fom": ("shell_flux", 1, "track-length flux of the graphite shell (30-60 cm)"),
        "more": [("leakage", 0, "leakage current at r = 70 cm"),
                 ("shell_flux", 2, "track-length flux of the borated shell (60-70 cm)")],
        "groups": 0, "prof": "",
    },
    "slab_1g": {
        "desc": "slab_1g: 1-group 20 cm slab, sigma_t 1, c 0.5, inward plane source, 100-bin flux",
        "histories": 1_000_000,
        "fom": ("reflection", 0, "reflected current at x = 0"),
        "more": [("transmission", 0, "transmitted current at x = 20 cm (~1e-9: unresolved)"),
                 ("slab", 0, "flux of the first 0.2 cm cell")],
        "groups": 0, "prof": "slab_1g/",
    },
    "mg_deep_slab": {
        "desc": "mg_deep_slab: 30-group 100 cm slab, 5 regions, importance 2^r, wr 0.25 / ws 1, group-1 plane source",
        "histories": 100_000_000,
        "fom": ("reflected", 0, "reflected current at x = 0"),
        "more": [("transmitted", 29, "group-30 transmitted current at x = 100 cm (unresolved)")],
        "groups": 30, "prof": "mg_deep_slab/",
    },
    "mg_layered_slab": {
        "desc": "mg_layered_slab: 16 x 1 cm one-group layers, sigma_t ~ U[0.5,2], c ~ U[0.3,0.95], inward plane source, transmitted + reflected current",
        "histories": 10_000_000,
        "fom": ("reflected", 0, "reflected current at x = 0"),
        "more": [("transmitted", 0, "transmitted current at x = 16 cm (~5e-9: unresolved)")],
        "groups": 1, "prof": "mg_layered_slab/",
    },
}


def make_workload(tmp: str, histories: int, workload: str = "ce_sphere") -> str:
    from mcgpu import workloads as W
    d = os.path.join(tmp, workload)
    if workload == "ce_sphere":
        W.ce_sphere(d, samples=histories)
    elif workload == "slab_1g":
        W.slab_1g(d, samples=histories)
    elif workload == "mg_deep_slab":
        W.mg_deep_slab(d, samples=histories)
    elif workload == "mg_layered_slab":
        W.mg_layered_slab(d, samples=histories, detectors="reflected")
    else:
        raise ValueError(workload)
    return d


def _xs_dir(d):
    x = os.path.join(d, "xs_library")
    return x if os.path.isdir(x) else None


def _traffic_key(leg, mode, tuned):
    """Key of the dominant kernel in profiles/traffic.json."""
    if mode != "event":
        return leg["prof"] + mode
    if tuned and tuned.get("kernel") == 2:
        return leg["prof"] + "event:k_track:%d" % tuned["blocks_per_sm"]   # by CTAs per SM
    if tuned and tuned.get("kernel") == 3:
        return leg["prof"] + "event:k_ev"
    return leg["prof"] + "event:k_event"


def _ncu_traffic():
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    and warp instructions per history of the dominant kernel of each
    workload, from the committed ncu captures summarised in profiles/."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except OSError:
        return None


def _issue_roofline(prof, leg, tuned, hist_per_s, clocks, sms):
    """The kernel against its issue bound: warp instructions per history
    (smsp__inst_executed.sum of the committed ncu capture of the same
    workload and launch shape) x histories/s, against 4 warp schedulers per
    SM, each issuing one instruction per cycle, at the SM clock sampled
    during the timed region; None when no capture of this shape is
    committed."""
    if not prof or not tuned or tuned.get("kernel") != 2:
        return None
    ipt = prof.get(leg["prof"] + "issue:k_track:%d" % tuned["blocks_per_sm"])
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not ipt or not mhz:
        return None
    peak = sms * 4 * mhz * 1e6
    achieved = ipt * hist_per_s
    thr = prof.get(leg["prof"] + "threads:k_track:%d" % tuned["blocks_per_sm"])
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "warp_instructions_per_history": ipt,
            "warp_execution_efficiency": thr / 32.0 if thr else None,
            "peak_source": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (sampled)"}


def _alg_bytes(leg, cnt):
    """Algorithmic bytes of the counters (continuous energy: 16 B per
    nuclide lookup at a flight -- sigma_s, sigma_c at two grid points in
    FP32 -- and 16 B per tally update, one FP64 read-modify-write;
    multigroup: 4 B per cross-section value, 4 B per probe of the
    ceil(log2 G)-step scatter-CDF bisection at each collision, 16 B per
    tally update)."""
    if leg["groups"] == 0:
        return 16 * cnt.get("nuc_lookups", 0) + 16 * cnt.get("tally_updates", 0)
    probes = math.ceil(math.log2(leg["groups"])) if leg["groups"] > 1 else 0
    return (4 * cnt.get("xs_evals", 0) + 4 * probes * cnt.get("collisions", 0)
            + 16 * cnt.get("tally_updates", 0))


def _tally_R(prob, name, b):
    m, s, _, _ = prob.tally(prob.names.index(name))
    return float(m[b]), (float(s[b] / m[b]) if m[b] != 0 else None)


# ----------------------------------------------------------------------------
# CPU oracle timing (cpu_baseline and --impl reference)
# ----------------------------------------------------------------------------
def _oracle_worker(args):
    d, first, n, seed = args
    from oracle import problem as OP
    pb = OP.load(d, xs_dir=_xs_dir(d))
    t0 = time.perf_counter()
    r = OP.run(pb, n=n, seed=seed, first=first)
    return time.perf_counter() - t0, r.status


def cpu_oracle_rate(d: str, n_per_proc: int, procs: int, first: int = 0):
    """histories/s of the CPU oracle with procs processes on disjoint ranges."""
    from oracle import problem as OP
    OP.build()
    ctx = mp.get_context("spawn")
    jobs = [(d, first + i * n_per_proc, n_per_proc, SEED) for i in range(procs)]
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_worker, jobs)
    wall = time.perf_counter() - t0
    busy = max(t for t, _ in res)
    return procs * n_per_proc / busy, wall


def cpu_oracle_sample(d: str, seconds: float, first: int):
    """One core: the oracle on growing history counts until one run takes
    about `seconds`; returns (histories/s, histories of that run)."""
    from oracle import problem as OP
    OP.build()
    pb = OP.load(d, xs_dir=_xs_dir(d))
    n = 200
    while True:
        t0 = time.perf_counter()
        OP.run(pb, n=n, seed=SEED, first=first)
        dt = time.perf_counter() - t0
        if dt >= 0.8 * seconds or n >= 50_000_000:
            return n / dt, n
        n = int(n * min(20.0, max(2.0, seconds / max(dt, 1e-3))))


def cpu_batch_sample(specs, seconds: float, procs: int = 1, start: int = 0, cap: int = 20_000):
    """The CPU oracle on problems of a batch taken in a seeded random order
    from position `start` (each run for min(histories, cap) histories), with
    `procs` processes, until about `seconds` of CPU time per process.  The
    batch's histories per problem are drawn independently of its geometry,
    so the batch's CPU time on one core is estimated as its total histories
    times the sampled problems' mean CPU time per history, and the problems,
    being independent, spread over `procs` cores.  Returns (histories/s of
    the whole batch on `procs` cores, problems sampled, histories run)."""
    import numpy as np
    from oracle import problem as OP
    OP.build()
    order = np.random.default_rng(SEED).permutation(len(specs))
    order = np.concatenate([order[start % len(order):], order[:start % len(order)]])
    per_hist, busy, ran, k = [], 0.0, 0, 0
    pool = mp.get_context("spawn").Pool(procs) if procs > 1 else None
    try:
        while busy < seconds * procs and k < len(order):
            chunk = order[k:k + 2 * procs]
            k += len(chunk)
            jobs = [(specs[i][0], 0, int(min(specs[i][1], cap)), SEED) for i in chunk]
            res = pool.map(_oracle_worker, jobs, chunksize=1) if pool else [_oracle_worker(j) for j in jobs]
            for j, (dt, _) in zip(jobs, res):
                per_hist.append(dt / j[2])
                busy += dt
                ran += j[2]
    finally:
        if pool:
            pool.close()
            pool.join()
    total = sum(h for _, h in specs)
    t_one_core = total * statistics.mean(per_hist)
    return total / (t_one_core / procs), len(per_hist), ran


def reference_batch_arm(a):
    """The batch on the host cores: the reference runs one Simulator per
    problem, so the problems spread over one oracle process per core; each
    step samples about ref-seconds of CPU time per process (cpu_batch_sample)."""
    from mcgpu import workloads as W
    procs = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        specs = W.batch_shields(tmp, n_problems=a.batch_problems)
        if a.warmup:
            cpu_batch_sample(specs, 0.2, procs, start=len(specs) // 2)
        rates, sampled, ran = [], 0, 0
        for k in range(a.steps):
            r, s_k, n_k = cpu_batch_sample(specs, a.ref_seconds, procs, start=k * 977)
            rates.append(r)
            sampled += s_k
            ran += n_k
    total = sum(h for _, h in specs)
    v = statistics.mean(rates)
    sample = (f"{sampled} problems of the batch in a seeded random order over {a.steps} steps, each run for "
              f"min(its histories, 20000) histories ({ran} in all) through the C oracle (restated reference "
              f"history loop, FP64), one process per core; the batch's CPU time is its {total} histories times "
              "the sampled mean CPU time per history, divided over the cores")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "histories/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * total / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"batch_shields: {len(specs)} MG slab/sphere shields, {total} histories, "
                                   "one problem at a time per host core",
                       "l2": "tables are L2-resident by design"},
            "cpu_baseline": {"value": v, "unit": "histories/s", "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def reference_arm(a):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    if a.workload == "batch":
        return reference_batch_arm(a)
    leg = LEGS[a.workload]
    procs = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        d = make_workload(tmp, a.histories or leg["histories"], a.workload)
        # bounded sample per step: the per-process history count is scaled so
        # that one step takes a few seconds of CPU time
        rate1, _ = cpu_oracle_sample(d, 1.0, first=10**9)
        n_per = a.ref_histories_per_proc or max(100, int(rate1 * a.ref_seconds))
        for w in range(max(0, min(a.warmup, 1))):
            cpu_oracle_rate(d, max(100, n_per // 10), procs, first=10**9)
        rates = []
        for k in range(a.steps):
            r, _ = cpu_oracle_rate(d, n_per, procs, first=k * procs * n_per)
            rates.append(r)
    v = statistics.mean(rates)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "histories/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * procs * n_per / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": leg["desc"], "histories_per_step": procs * n_per,
                       "l2": "tables are L2-resident by design"},
            "cpu_baseline": {"value": v, "unit": "histories/s", "cores": procs, "kind": "port",
                             "sample": f"{procs} processes x {n_per} histories per step, "
                                       "C oracle (restated reference history loop, FP64)"},
            "e2e": {"value": v, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def gpu_arm(a):
    rank, world, local = _env_rank()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("nccl")
    import build as B
    B.build()
    import mcgpu
    from mcgpu import parallel
    import numpy as np

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    if a.workload == "batch":
        return batch_arm(a, mcgpu, torch, flush, rank, world, dist)
    leg = LEGS[a.workload]
    H = a.histories or leg["histories"]
    with tempfile.TemporaryDirectory() as tmp:
        d = make_workload(tmp, H, a.workload)
        prob = mcgpu.Problem(d, _xs_dir(d))
        run_kw = {}
        if a.mode != "event":
            tuned = None
        elif a.kernel == "auto":
            tuned = prob.autotune(sample=min(H, 1_000_000), seed=SEED + 17)
        else:
            kmap = {"tile": 1, "thread": 2, "bank": 3}
            if a.blocks_per_sm is None:
                a.blocks_per_sm = {"tile": 2, "thread": 8, "bank": 0}[a.kernel]
            tuned = {"kernel": kmap[a.kernel], "blocks_per_sm": a.blocks_per_sm,
                     "bank_capacity": a.tile if a.kernel in ("tile", "bank") else 0}
            run_kw = dict(kernel=tuned["kernel"])
            if a.blocks_per_sm:
                run_kw["blocks_per_sm"] = a.blocks_per_sm
            if a.kernel in ("tile", "bank") and a.tile:
                run_kw["bank_capacity"] = a.tile
        base = rank * (a.steps + a.warmup + a.e2e_steps + 1) * H
        for w in range(a.warmup):
            prob.reset()
            prob.run(n=H, first=base + w * H, seed=SEED, mode=a.mode, **run_kw)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        sampler = ClockSampler(local)
        sampler.start()
        dev_ms, transport_ms, launches = 0.0, 0.0, 0
        cnt_sum = {}
        fom_steps = {}
        wall0 = time.perf_counter()
        for k in range(a.steps):
            flush.zero_()
            torch.cuda.synchronize()
            prob.reset()
            c = prob.run(n=H, first=base + (a.warmup + k) * H, seed=SEED, mode=a.mode, **run_kw)
            dev_ms += c["total_ms"]
            transport_ms += c["transport_ms"]
            launches += c["launches"]
            for key in ("flights", "collisions", "crossings", "tally_updates", "nuc_lookups",
                        "xs_evals", "particles", "freegas_iters", "splits"):
                cnt_sum[key] = cnt_sum.get(key, 0) + c[key]
            T = c["total_ms"] * 1e-3
            for (name, b, _) in [leg["fom"]] + leg["more"]:
                mean, R = _tally_R(prob, name, b)
                fom_steps.setdefault((name, b), []).append((mean, R, 1.0 / (R * R * T) if R else None))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        clocks = sampler.stop()
        # the last timed step's sums, merged over the ranks in rank order
        merged = None
        if dist:
            _, _, s_last, q_last = prob.all_tallies()
            ms, mq = parallel.gather_sums(s_last, q_last, dist, device="cuda")
            if rank == 0:
                mean_m, sig_m = parallel.statistics(ms, mq, world * H)
                off = sum(prob.sizes[:prob.names.index(leg["fom"][0])]) + leg["fom"][1]
                mean0, R0 = _tally_R(prob, leg["fom"][0], leg["fom"][1])
                z = abs(mean_m[off] - mean0) / (mean0 * R0) if R0 else None
                merged = {"histories": world * H, "tally": leg["fom"][2], "mean": float(mean_m[off]),
                          "R": float(sig_m[off] / mean_m[off]) if mean_m[off] else None,
                          "rank0_mean": mean0, "rank0_R": R0, "z_vs_rank0": z,
                          "merge": "per-bin (sum, sum of squares) of every rank, added in rank order"}
        # e2e through the C ABI: upload tables (pinned host -> device), run,
        # read every tally back
        e2e_t = 0.0
        h2d = prob.table_bytes()
        d2h = 0
        for k in range(a.e2e_steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prob.upload()
            prob.reset()
            prob.run(n=H, first=base + (a.warmup + a.steps + k) * H, seed=SEED, mode=a.mode, **run_kw)
            tot = prob.all_tallies()
            e2e_t += time.perf_counter() - t0
            d2h = int(sum(x.nbytes for x in tot[2:]))
        # the plain FP64 GPU history path on the same problem, run until its
        # FOM tally reaches R <= 1 % as well (after the timed region, rank 0)
        plain = None
        if a.mode == "event" and a.plain and rank == 0:
            name, b, what = leg["fom"]
            prob.reset()
            pilot = min(H, 200_000)
            prob.run(n=pilot, first=10**11, seed=SEED, mode="plain")
            _, Rp = _tally_R(prob, name, b)
            Hp = int(pilot * (Rp / 0.009) ** 2) if Rp else H
            Hp = max(pilot, min(Hp, a.plain_max_histories))
            prob.reset()
            cp = prob.run(n=Hp, first=10**11 + pilot, seed=SEED, mode="plain")
            mp_, Rp = _tally_R(prob, name, b)
            Tp = cp["total_ms"] * 1e-3
            plain = {"value": Hp / Tp, "unit": "histories/s", "histories": Hp, "R": Rp,
                     "fom": 1.0 / (Rp * Rp * Tp) if Rp else None, "tally": what,
                     "note": "MC_FP64_PLAIN on the same workload (FP64 tracking, native FP64 math), "
                             "histories chosen so that the FOM tally reaches R <= 1 %"}
        prob.close()

    value_local = a.steps * H / (dev_ms * 1e-3)
    step_ms = dev_ms / a.steps
    if dist:
        t = torch.tensor([dev_ms, e2e_t], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms_max, e2e_max = float(t[0]), float(t[1])
        dist.destroy_process_group()
    else:
        dev_ms_max, e2e_max = dev_ms, e2e_t
    if rank != 0:
        return 0
    value = world * a.steps * H / (dev_ms_max * 1e-3)
    e2e_value = world * a.e2e_steps * H / e2e_max if a.e2e_steps else None
    peaks, peak_kind = _measured_peaks()
    alg_bytes = _alg_bytes(leg, cnt_sum)
    achieved = alg_bytes / (transport_ms * 1e-3) / 1e9 if transport_ms > 0 else 0.0
    traffic = _ncu_traffic()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    l2_peak = _l2_read_gbs(torch)
    cpu = None
    if a.cpu_baseline:
        with tempfile.TemporaryDirectory() as tmp:
            d = make_workload(tmp, H, a.workload)
            r1, n1 = cpu_oracle_sample(d, a.cpu_seconds, first=10**10)
        cpu = {"value": r1, "unit": "histories/s", "cores": 1, "kind": "port",
               "sample": f"{n1} histories of the same workload through the C oracle "
                         "(restated reference history loop, FP64), one core"}

    def fom_entry(key, what):
        rows = fom_steps.get(key, [])
        foms = [f for _, _, f in rows if f]
        Rs = [R for _, R, _ in rows if R]
        return {"value": statistics.mean(foms) if foms else None, "unit": "1/s", "tally": what,
                "R": statistics.mean(Rs) if Rs else None}

    fom_main = fom_entry(leg["fom"][:2], leg["fom"][2])
    fom_main["tallies"] = [fom_entry((n_, b_), w_) for n_, b_, w_ in leg["more"]]
    line = {
        "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"event": "f32", "plain": "f64", "replay": "f64"}[a.mode],
        "dtype_detail": {"event": "f32 tracking, f64 tally accumulation", "plain": "f64",
                         "replay": "f64, the reference's operation order"}[a.mode],
        "data": "synthetic",
        "config": {"workload": leg["desc"], "histories_per_step": H, "mode": a.mode,
                   "launch_shape": _shape(tuned),
                   "l2": "flushed (256 MiB write) before every timed step; cross-section tables L2-resident by design",
                   "parallelism": f"dp{world} (disjoint history ranges)"},
        "fom": fom_main,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": (traffic or {}).get(_traffic_key(leg, a.mode, tuned)),
                     "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs",
                     "algorithmic_bytes_per_step": alg_bytes / a.steps,
                     "kernel_ms_per_step": transport_ms / a.steps},
        "roofline_issue": _issue_roofline(traffic, leg, tuned, value_local, clocks,
                                          torch.cuda.get_device_properties(0).multi_processor_count),
        "roofline_l2": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                        "frac": achieved / l2_peak if l2_peak else None,
                        "peak_source": "measured in this run: one reduction kernel reading a 32 MiB L2-resident buffer 64 times"},
        "counters_per_step": {k: v / a.steps for k, v in cnt_sum.items()},
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "histories/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "wall_s_timed": wall,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if plain:
        fom_m = line["fom"]["value"]
        plain["fom_ratio"] = fom_m / plain["fom"] if (fom_m and plain["fom"]) else None
        plain["matched_R"] = bool(line["fom"]["R"] and plain["R"] and line["fom"]["R"] <= 0.01
                                  and plain["R"] <= 0.01)
        line["plain_fp64"] = plain
    if merged:
        line["merged"] = merged
    print(json.dumps(line))
    return 0


def batch_arm(a, mcgpu, torch, flush, rank, world, dist):
    """Config of 4096 uneven multigroup shields in one persistent launch."""
    from mcgpu import workloads as W
    import numpy as np
    with tempfile.TemporaryDirectory() as tmp:
        specs = W.batch_shields(tmp, n_problems=a.batch_problems)
        probs = [mcgpu.Problem(d) for d, _ in specs]
        hist = [h for _, h in specs]
        b = mcgpu.Batch(probs, hist)
        run_kw = {}
        if a.kernel == "auto":
            tuned = b.autotune(seed=SEED + 17, fraction=0.05)
        else:   # a fixed shape (profiling runs)
            mb = a.blocks_per_sm if a.blocks_per_sm is not None else (2 if a.kernel == "tile" else 8)
            tuned = {"kernel": 1 if a.kernel == "tile" else 2, "blocks_per_sm": mb,
                     "bank_capacity": a.tile if a.kernel == "tile" else 0}
            run_kw = dict(kernel=tuned["kernel"], blocks_per_sm=mb)
            if a.kernel == "tile":
                run_kw["bank_capacity"] = a.tile
        for w in range(a.warmup):
            for p in probs:
                p.reset()
            b.run(seed=SEED + 1000 + w, **run_kw)
        torch.cuda.synchronize()
        sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        sampler.start()
        ms, launches, foms = 0.0, 0, []
        cnt_sum = {}
        for k in range(a.steps):
            flush.zero_()
            torch.cuda.synchronize()
            for p in probs:
                p.reset()
            c = b.run(seed=SEED + k, **run_kw)
            ms += c["total_ms"]
            launches += c["launches"]
            for key in ("flights", "collisions", "crossings", "tally_updates", "xs_evals", "particles"):
                cnt_sum[key] = cnt_sum.get(key, 0) + c[key]
        clocks = sampler.stop()
        T = ms / a.steps * 1e-3
        for p in probs:
            m, s, _, _ = p.tally(0)
            tot = float(np.sum(m))
            if tot > 0:
                err = float(np.sqrt(np.sum(s ** 2))) / tot
                foms.append(1.0 / (err * err * T))
        # e2e through the C ABI: every problem's tables uploaded again from
        # pinned host memory, the tallies cleared, the batch run, every
        # problem's tallies read back (the batch-wide calls: one wait each)
        e2e_t = 0.0
        h2d = int(sum(p.table_bytes() for p in probs))
        d2h = 0
        for k in range(a.e2e_steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.upload()
            b.reset()
            b.run(seed=SEED + 100 + k, **run_kw)
            tot = b.tallies()
            e2e_t += time.perf_counter() - t0
            d2h = int(sum(x.nbytes for x in tot[2:]))
        b.close()
        for p in probs:
            p.close()
        cpu = None
        if a.cpu_baseline:
            r1, s1, n1 = cpu_batch_sample(specs, a.cpu_seconds, 1)
            cpu = {"value": r1, "unit": "histories/s", "cores": 1, "kind": "port",
                   "sample": f"{s1} problems of the batch in a seeded random order, each run for min(its "
                             f"histories, 20000) histories ({n1} in all) through the C oracle (restated "
                             "reference history loop, FP64), one core; the batch's CPU time is its histories "
                             "times the sampled mean CPU time per history"}
    total = sum(hist)
    peaks, peak_kind = _measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # multigroup: one 4-byte table value per cross-section evaluation (the
    # scatter-CDF probes are not counted), one FP64 update per tally update
    alg_bytes = (4 * cnt_sum.get("xs_evals", 0) + 16 * cnt_sum.get("tally_updates", 0)) / a.steps
    achieved = alg_bytes / T / 1e9
    line = {"metric": METRIC, "value": total / T, "unit": "histories/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": T * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "dtype_detail": "f32 tracking, f64 tally accumulation",
            "data": "synthetic",
            "config": {"workload": f"batch_shields: {len(hist)} MG slab/sphere shields, {total} histories, "
                                   "one persistent launch from a CUDA graph",
                       "launch_shape": _shape(tuned),
                       "l2": "flushed (256 MiB write) before every timed step"},
            "batch_latency_ms": T * 1e3,
            "fom_per_problem": {"median": float(np.median(foms)), "min": float(np.min(foms)),
                                "max": float(np.max(foms)), "unit": "1/s",
                                "tally": "total leakage, R over the group bins, T = whole-batch latency"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak if peak else None, "traffic": None,
                         "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs",
                         "algorithmic_bytes_per_step": alg_bytes},
            "roofline_issue": _issue_roofline(_ncu_traffic(), {"prof": "batch/" if len(hist) == 4096 else "batch%d/" % len(hist)},
                                              tuned, total / T, clocks,
                                              torch.cuda.get_device_properties(0).multi_processor_count),
            "counters_per_step": {k: v / a.steps for k, v in cnt_sum.items()},
            "e2e": {"value": total * a.e2e_steps / e2e_t if a.e2e_steps else None, "unit": "histories/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clocks, "gpu_launches": launches}
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="event", choices=["event", "plain", "replay"])
    ap.add_argument("--workload", default="ce_sphere", choices=list(LEGS) + ["batch"])
    ap.add_argument("--batch-problems", type=int, default=4096)
    ap.add_argument("--histories", type=int, default=0, help="histories per step (0: the workload's own)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "tile", "thread", "bank"],
                    help="event mode: autotuned, or a fixed kernel (no autotuning launches; for profiling)")
    ap.add_argument("--blocks-per-sm", type=int, default=None,
                    help="with --kernel: resident CTAs per SM (tile: 2-4, default 2; thread: 4, 6, 7, 8, default 8)")
    ap.add_argument("--tile", type=int, default=0, help="with --kernel tile / bank: particles per tile / bank")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU time of the one-core oracle sample (cpu_baseline)")
    ap.add_argument("--no-plain", dest="plain", action="store_false",
                    help="skip the plain FP64 comparison run")
    ap.add_argument("--plain-max-histories", type=int, default=20_000_000)
    ap.add_argument("--ref-histories-per-proc", type=int, default=0,
                    help="reference arm: histories per process per step (0: ~ref-seconds of CPU time)")
    ap.add_argument("--ref-seconds", type=float, default=3.0)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3) if a.impl == "gb300" else a.warmup
    if a.impl == "reference":
        return reference_arm(a)
    return gpu_arm(a)


if __name__ == "__main__":
    sys.exit(main())
