"""Build libmcgpu.so (the CUDA library behind include/mcgpu.h) in-tree.

Compiles every translation unit in parallel for sm_103a only and links one
shared library into mcgpu/libmcgpu.so.  Flags that matter for results:

  * host C++ uses -ffp-contract=off so that set-up arithmetic (plane
    coefficients, lethargy grids) gives the same bits on x86-64 and aarch64;
  * mc_history.cu (FP64 replay / plain) uses -fmad=false so that no multiply
    and add are fused and the replay matches the CPU oracle bit for bit;
  * the mixed-precision kernels keep FMA contraction and use approximate
    FP32 division and square root with denormals flushed to zero (they are
    not bit-exact by design; the statistical tests against FP64 replay and
    the analytic slab bound the effect).

    python mc-old_gb300/build.py [-v] [--clean]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "mcgpu", "libmcgpu.so")
EXE = os.path.join(HERE, "mcgpu", "mcgpu_run")      # MC.exe counterpart (csrc/mc_main.cpp)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, kind): host = g++, fp64 = nvcc without FMA contraction, fast = nvcc
SOURCES = [
    ("mc_xml.cpp", "host"),
    ("mc_problem.cpp", "host"),
    ("mc_engine.cpp", "host"),
    ("mc_api.cpp", "host"),
    ("mc_report.cpp", "host"),
    ("mc_evtables.cpp", "host"),
    ("mc_api_batch.cpp", "host"),
    ("mc_lr.cpp", "host"),
    ("mc_history.cu", "fp64"),
    ("mc_event.cu", "fast"),
    ("mc_event_ce.cu", "fast"),
    ("mc_event_mg.cu", "fast"),
    ("mc_event_all.cu", "fast"),
    ("mc_bank.cu", "fast"),
    ("mc_noalloc.cu", "fp64"),
    ("mc_exact.cu", "fp64"),
]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "mcgpu.h"))
    return hs


def _cmd(src: str, kind: str, obj: str):
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if kind == "host":
        return ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
                "-Wno-unused-parameter", "-I", os.path.join(CUDA, "include")] + inc + ["-c", src, "-o", obj]
    cmd = [NVCC] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                           "-Xptxas", "-warn-spills"] + inc
    if kind == "fp64":
        cmd += ["-fmad=false"]
    if kind == "fast":
        # FP32 tracking: approximate division and square root (a few ulp),
        # denormals flushed; the statistical tests bound the effect
        cmd += ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
    return cmd + ["-c", src, "-o", obj]


def build(verbose: bool = False, clean: bool = False) -> str:
    if clean and os.path.isdir(BUILD):
        shutil.rmtree(BUILD)
    os.makedirs(BUILD, exist_ok=True)
    newest_header = max(os.path.getmtime(h) for h in _headers())
    jobs = []
    objs = []
    for name, kind in SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name + ".o")
        objs.append(obj)
        if (not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src)
                or os.path.getmtime(obj) < newest_header
                or os.path.getmtime(obj) < os.path.getmtime(__file__)):
            jobs.append(_cmd(src, kind, obj))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                print(" ".join(cmd), file=sys.stderr)
                print(r.stdout + r.stderr, file=sys.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"compile failed: {cmd[-3]}")
    if jobs or not os.path.exists(LIB):
        link = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(link, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(link), file=sys.stderr)
            print(r.stdout + r.stderr, file=sys.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    main_src = os.path.join(CSRC, "mc_main.cpp")
    if (not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(LIB)
            or os.path.getmtime(EXE) < os.path.getmtime(main_src)):
        exe = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), main_src,
               "-L", os.path.dirname(LIB), "-lmcgpu", "-Wl,-rpath,$ORIGIN", "-o", EXE]
        r = subprocess.run(exe, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(exe), file=sys.stderr)
            print(r.stdout + r.stderr, file=sys.stderr)
        if r.returncode != 0:
            raise RuntimeError("driver link failed")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--clean", action="store_true")
    a = ap.parse_args()
    print(build(verbose=a.verbose, clean=a.clean))
