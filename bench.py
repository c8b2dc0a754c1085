"""Benchmark of the fixed-source particle-history path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode event|plain|replay]
                    [--histories H] [--impl reference]

Workload: the continuous-energy spherical shield (three shells: water-like
H1/O16 0-30 cm, graphite 30-60 cm, borated graphite 60-70 cm; 20,000-point
log-uniform synthetic tables for five nuclides; isotropic 2 MeV point source;
leakage current, 50-bin lethargy spectrum in the outer shell, per-shell flux).
One step = one mc_run over H histories (default 10^7, the workload's size) on
a fresh history range.  Inputs are synthetic (numpy PCG64 seeded, see
mcgpu/workloads.py).  The cross-section tables (0.8 MB FP32 / 1.6 MB FP64)
are L2-resident by design; L2 is flushed between timed steps with a 256 MiB
write.

value      histories/s over all ranks, device time (CUDA events on the
           library's stream) summed over the K timed steps, max over ranks.
fom        1/(R^2 T) for the leakage tally (R its relative error after one
           step, T the step time).
e2e        the same metric through the C ABI from the host: per step, the
           problem tables re-uploaded from pinned host memory
           (mc_problem_upload), mc_run, and every tally read back to host
           buffers (mc_tally_read); wall clock.
roofline   the transport kernels against HBM: algorithmic bytes per run =
           16 B x (nuclide lookups at flights) + 16 B x (tally bin updates)
           (XS lookup: sigma_s, sigma_c at two grid points in FP32 per
           nuclide; tally: one FP64 read-modify-write), from the device
           counters, over the transport kernels' CUDA-event time; peak =
           MEASURED_PEAKS.json hbm_gbs; traffic from the committed ncu summary.
roofline_l2  the same algorithmic bytes against an L2 read bandwidth measured
           in the run (the tables are L2-resident).
roofline_issue  the kernel against its issue bound: warp instructions per
           history from the committed ncu capture of the same launch shape
           x histories/s, over 4 schedulers per SM x the sampled SM clock.
cpu_baseline  the CPU oracle (a C restatement of the reference's history loop)
           on the host cores, on a bounded sample of the same workload.
plain_fp64 the plain FP64 GPU history path (MC_FP64_PLAIN) on the same
           workload after the timed region: histories/s, FOM and the
           mixed / plain FOM ratio.

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
    (tile particles per CTA), kernel 2 = one particle per thread."""
    if not tuned:
        return None
    if tuned.get("kernel") == 2:
        return {"kernel": "per-thread (k_track)", "blocks_per_sm": tuned["blocks_per_sm"]}
    return {"kernel": "tile (k_event)", "tile": tuned["bank_capacity"], "blocks_per_sm": tuned["blocks_per_sm"]}


def _traffic_key(mode, tuned):
    """Key of the dominant kernel in profiles/traffic.json."""
    if mode != "event":
        return mode
    if tuned and tuned.get("kernel") == 2:
        return "event:k_track:%d" % tuned["blocks_per_sm"]   # by CTAs per SM
    return "event:k_event"


def _ncu_traffic():
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    of the dominant kernel on this workload, from the committed ncu capture
    summarised in profiles/; None if absent."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except OSError:
        return None


def _issue_roofline(prof, tuned, hist_per_s, clocks, sms):
    """The kernel against its issue bound: warp instructions per history
    (smsp__inst_executed.sum of the committed full ncu capture of the same
    launch shape) x histories/s, against 4 warp schedulers per SM, each
    issuing one instruction per cycle, at the SM clock sampled during the
    timed region; None when no capture of this shape is committed."""
    if not prof or not tuned or tuned.get("kernel") != 2:
        return None
    ipt = prof.get("issue:k_track:%d" % tuned["blocks_per_sm"])
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not ipt or not mhz:
        return None
    peak = sms * 4 * mhz * 1e6
    achieved = ipt * hist_per_s
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "warp_instructions_per_history": ipt,
            "peak_source": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (sampled)"}


def make_workload(tmp: str, histories: int) -> str:
    from mcgpu import workloads as W
    d = os.path.join(tmp, "ce_sphere")
    W.ce_sphere(d, samples=histories)
    return d


# ----------------------------------------------------------------------------
# CPU oracle timing (cpu_baseline and --impl reference)
# ----------------------------------------------------------------------------
def _oracle_worker(args):
    d, first, n, seed = args
    from oracle import problem as OP
    pb = OP.load(d, xs_dir=os.path.join(d, "xs_library"))
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


def reference_arm(a):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    procs = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        d = make_workload(tmp, a.histories)
        # bounded sample per step: ~2 s of CPU work per process
        n_per = a.ref_histories_per_proc
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
            "config": {"workload": WORKLOAD, "histories_per_step": procs * n_per,
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
    import numpy as np

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    if a.workload == "batch":
        return batch_arm(a, mcgpu, torch, flush, rank, world, dist)
    with tempfile.TemporaryDirectory() as tmp:
        d = make_workload(tmp, a.histories)
        prob = mcgpu.Problem(d, os.path.join(d, "xs_library"))
        H = a.histories
        run_kw = {}
        if a.mode != "event":
            tuned = None
        elif a.kernel == "auto":
            tuned = prob.autotune(sample=min(H, 1_000_000), seed=SEED + 17)
        else:
            if a.blocks_per_sm is None:
                a.blocks_per_sm = 2 if a.kernel == "tile" else 8
            tuned = {"kernel": 1 if a.kernel == "tile" else 2, "blocks_per_sm": a.blocks_per_sm,
                     "bank_capacity": a.tile if a.kernel == "tile" else 0}
            run_kw = dict(kernel=tuned["kernel"], blocks_per_sm=a.blocks_per_sm)
            if a.kernel == "tile":
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
        fom = []
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
                        "xs_evals", "particles", "freegas_iters"):
                cnt_sum[key] = cnt_sum.get(key, 0) + c[key]
            m, s, _, _ = prob.tally(prob.names.index("leakage"))
            if m[0] > 0:
                fom.append(1.0 / ((s[0] / m[0]) ** 2 * (c["total_ms"] * 1e-3)))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
        clocks = sampler.stop()
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
        # the plain FP64 GPU history path on the same problem, for the
        # metric's "vs plain FP64" (after the timed region, rank 0 only)
        plain = None
        if a.mode == "event" and a.plain_histories > 0 and rank == 0:
            Hp = a.plain_histories
            prob.reset()
            prob.run(n=min(Hp, 20000), first=10**11, seed=SEED, mode="plain")
            prob.reset()
            cp = prob.run(n=Hp, first=10**11 + Hp, seed=SEED, mode="plain")
            mp, sp, _, _ = prob.tally(prob.names.index("leakage"))
            Tp = cp["total_ms"] * 1e-3
            fom_p = 1.0 / ((sp[0] / mp[0]) ** 2 * Tp) if mp[0] > 0 else None
            plain = {"value": Hp / Tp, "unit": "histories/s", "histories": Hp, "fom": fom_p,
                     "note": "MC_FP64_PLAIN on the same workload: FP64 tracking, native FP64 math"}
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
    alg_bytes = 16 * cnt_sum.get("nuc_lookups", 0) + 16 * cnt_sum.get("tally_updates", 0)
    achieved = alg_bytes / (transport_ms * 1e-3) / 1e9 if transport_ms > 0 else 0.0
    traffic = _ncu_traffic()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    l2_peak = _l2_read_gbs(torch)
    cpu = None
    if a.cpu_baseline:
        with tempfile.TemporaryDirectory() as tmp:
            d = make_workload(tmp, H)
            n_per = a.cpu_histories
            r1, _ = cpu_oracle_rate(d, n_per, 1, first=10**10)
        cpu = {"value": r1, "unit": "histories/s", "cores": 1, "kind": "port",
               "sample": f"{n_per} histories of the same workload through the C oracle "
                         "(restated reference history loop, FP64), one core"}
    line = {
        "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"event": "f32", "plain": "f64", "replay": "f64"}[a.mode],
        "dtype_detail": {"event": "f32 tracking, f64 tally accumulation", "plain": "f64",
                         "replay": "f64, the reference's operation order"}[a.mode],
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "histories_per_step": H, "mode": a.mode,
                   "launch_shape": _shape(tuned),
                   "l2": "flushed (256 MiB write) before every timed step; XS tables L2-resident by design",
                   "parallelism": f"dp{world} (disjoint history ranges)"},
        "fom": {"value": statistics.mean(fom) if fom else None, "unit": "1/s",
                "tally": "leakage current at r=70 cm, R after one step"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": (traffic or {}).get(_traffic_key(a.mode, tuned)),
                     "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs",
                     "algorithmic_bytes_per_step": alg_bytes / a.steps,
                     "kernel_ms_per_step": transport_ms / a.steps},
        "roofline_issue": _issue_roofline(traffic, tuned, value_local, clocks,
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
        line["plain_fp64"] = plain
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
            tuned = b.autotune(seed=SEED + 17, fraction=0.01)
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
        # pinned host memory, the batch run, every problem's tallies read back
        e2e_t = 0.0
        h2d = int(sum(p.table_bytes() for p in probs))
        d2h = 0
        for k in range(a.e2e_steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for p in probs:
                p.upload()
                p.reset()
            b.run(seed=SEED + 100 + k, **run_kw)
            d2h = 0
            for p in probs:
                tot = p.all_tallies()
                d2h += int(sum(x.nbytes for x in tot[2:]))
            e2e_t += time.perf_counter() - t0
        b.close()
        for p in probs:
            p.close()
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
            "counters_per_step": {k: v / a.steps for k, v in cnt_sum.items()},
            "e2e": {"value": total * a.e2e_steps / e2e_t if a.e2e_steps else None, "unit": "histories/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clocks, "gpu_launches": launches}
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
    ap.add_argument("--workload", default="ce_sphere", choices=["ce_sphere", "batch"])
    ap.add_argument("--batch-problems", type=int, default=4096)
    ap.add_argument("--histories", type=int, default=10_000_000)
    ap.add_argument("--kernel", default="auto", choices=["auto", "tile", "thread"],
                    help="event mode: autotuned, or a fixed kernel (no autotuning launches; for profiling)")
    ap.add_argument("--blocks-per-sm", type=int, default=None,
                    help="with --kernel: resident CTAs per SM (tile: 2-4, default 2; thread: 4, 6, 7, 8, default 8)")
    ap.add_argument("--tile", type=int, default=512)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-histories", type=int, default=4000)
    ap.add_argument("--plain-histories", type=int, default=500_000,
                    help="histories of the plain FP64 comparison run (0: skip)")
    ap.add_argument("--ref-histories-per-proc", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3) if a.impl == "gb300" else a.warmup
    if a.impl == "reference":
        return reference_arm(a)
    return gpu_arm(a)


if __name__ == "__main__":
    sys.exit(main())
