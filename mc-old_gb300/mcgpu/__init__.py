"""mcgpu -- Python host interface of the GB300 fixed-source library.

Two layers over the C ABI of include/mcgpu.h (loaded with ctypes from the
in-tree libmcgpu.so; there is no CPU fallback -- if the library or a CUDA
device is missing every call raises):

* ``Problem``: thin handle (load, run a history range in a mode, read tallies,
  counters, digests, write the report).
* ``Simulator``: the reference's interface for this path, same names and
  meaning as MC-old's ``Simulator`` (include/simulator.h:21-150):
  ``Simulator(io_dir)`` reads ``io_dir/input.xml`` (setup.cpp:30),
  ``start()`` runs ``Nsample`` histories (handler.cpp:11-48),
  ``Estimators[i].tally(j).mean / .uncer`` (Estimator.cpp:424-427),
  ``tally_size()`` (:429-432), ``Ntrack`` (general.cpp:76) and
  ``report(io_dir)`` (report.cpp:9-50, written as JSON).  Input errors raise
  ``InputError`` where the reference would print and exit.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcgpu.so")

MODES = {"replay": 0, "plain": 1, "event": 2}
STATUS = {0: "MC_OK", 1: "MC_ERR_INPUT", 2: "MC_ERR_CUDA", 3: "MC_ERR_OVERFLOW", 4: "MC_ERR_LOST",
          5: "MC_ERR_TIMEOUT", 6: "MC_ERR_NAN", 7: "MC_ERR_NOMEM", 8: "MC_ERR_ARG"}
DEFAULT_SEED = 0x4D43


class McError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class InputError(McError):
    pass


class Tune(ctypes.Structure):
    _fields_ = [("block", ctypes.c_uint32), ("grid_blocks", ctypes.c_uint32),
                ("stack_depth", ctypes.c_uint32), ("chunk", ctypes.c_uint32),
                ("bank_capacity", ctypes.c_uint32), ("record_digests", ctypes.c_uint32),
                ("blocks_per_sm", ctypes.c_uint32), ("kernel", ctypes.c_uint32),
                ("max_events", ctypes.c_uint32), ("refill", ctypes.c_uint32)]


class Counters(ctypes.Structure):
    _fields_ = [("flights", ctypes.c_uint64), ("collisions", ctypes.c_uint64),
                ("crossings", ctypes.c_uint64), ("tally_updates", ctypes.c_uint64),
                ("particles", ctypes.c_uint64), ("splits", ctypes.c_uint64),
                ("xs_evals", ctypes.c_uint64), ("freegas_iters", ctypes.c_uint64),
                ("nuc_lookups", ctypes.c_uint64), ("histories", ctypes.c_uint64),
                ("transport_ms", ctypes.c_double), ("fold_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("launches", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib() -> ctypes.CDLL:
    """Load libmcgpu.so (built by mc-old_gb300/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise McError(2, f"{LIB_PATH} is missing: build it with mc-old_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        P, u32, u64, st = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        L.mc_problem_load_xml.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(P)]
        L.mc_problem_free.argtypes = [P]
        L.mc_problem_upload.argtypes = [P]
        L.mc_problem_table_bytes.argtypes = [P, ctypes.POINTER(u64)]
        L.mc_run.argtypes = [P, u64, u64, u64, st, ctypes.POINTER(Tune)]
        L.mc_reset_tallies.argtypes = [P]
        L.mc_tally_count.argtypes = [P, ctypes.POINTER(u32)]
        L.mc_tally_size.argtypes = [P, u32, ctypes.POINTER(u64)]
        L.mc_estimator_name.argtypes = [P, u32, ctypes.c_char_p, ctypes.c_size_t]
        L.mc_tally_read.argtypes = [P, u32, P, P, P, P, u64]
        L.mc_counters_read.argtypes = [P, ctypes.POINTER(Counters)]
        L.mc_digests_read.argtypes = [P, P, u64]
        L.mc_nsample.argtypes = [P, ctypes.POINTER(u64)]
        L.mc_histories_run.argtypes = [P, ctypes.POINTER(u64)]
        L.mc_report.argtypes = [P, ctypes.c_char_p]
        L.mc_state_save.argtypes = [P, ctypes.c_char_p]
        L.mc_state_load.argtypes = [P, ctypes.c_char_p]
        L.mc_autotune.argtypes = [P, u64, u64, ctypes.POINTER(Tune)]
        L.mc_lr_params.argtypes = [P, P, u32]
        L.mc_forward.argtypes = [P, P, u64, u64, P, P]
        L.mc_backward.argtypes = [P, P, u64, u64, P, P]
        L.mc_backward_density.argtypes = [P, P, u64, u64, P, P, P, P]
        L.mc_batch_create.argtypes = [ctypes.POINTER(P), u32, ctypes.POINTER(u64), ctypes.POINTER(P)]
        L.mc_batch_run.argtypes = [P, u64, ctypes.POINTER(Tune)]
        L.mc_batch_counters.argtypes = [P, ctypes.POINTER(Counters)]
        L.mc_batch_autotune.argtypes = [P, u64, ctypes.c_double, ctypes.POINTER(Tune)]
        L.mc_batch_free.argtypes = [P]
        L.mc_batch_upload.argtypes = [P]
        L.mc_batch_reset.argtypes = [P]
        L.mc_batch_tally_read.argtypes = [P, P, P, P, P, u64]
        L.mc_batch_last_error.argtypes = [P]
        L.mc_batch_last_error.restype = ctypes.c_char_p
        L.mc_last_error.argtypes = [P]
        L.mc_last_error.restype = ctypes.c_char_p
        L.mc_exact_sums_read.argtypes = [P, P, u64]
        L.mc_exact_round.argtypes = [P, u64, P]
        L.mc_status_string.argtypes = [st]
        L.mc_status_string.restype = ctypes.c_char_p
        for f in ("mc_problem_load_xml", "mc_problem_free", "mc_problem_upload",
                  "mc_problem_table_bytes", "mc_run", "mc_reset_tallies",
                  "mc_tally_count", "mc_tally_size", "mc_estimator_name", "mc_tally_read",
                  "mc_counters_read", "mc_digests_read", "mc_nsample", "mc_histories_run",
                  "mc_report", "mc_state_save", "mc_state_load", "mc_autotune", "mc_lr_params", "mc_forward", "mc_backward", "mc_backward_density", "mc_batch_create", "mc_batch_run", "mc_batch_counters",
                  "mc_batch_autotune", "mc_batch_free", "mc_exact_sums_read", "mc_exact_round",
                  "mc_batch_upload", "mc_batch_reset", "mc_batch_tally_read"):
            getattr(L, f).restype = st
        _lib = L
    return _lib


EXACT_LIMBS = 68   # MC_EXACT_LIMBS


def exact_round(limbs) -> np.ndarray:
    """Nearest doubles of exact values ([..., EXACT_LIMBS] int64 limbs) by the
    library's mc_exact_round (host arithmetic)."""
    a = np.ascontiguousarray(limbs, np.int64)
    n = a.size // EXACT_LIMBS
    out = np.zeros(max(n, 1))
    st = lib().mc_exact_round(a.ctypes.data, n, out.ctypes.data)
    if st != 0:
        raise McError(st, "mc_exact_round")
    return out[:n].reshape(a.shape[:-1])


def make_tune(**kw) -> Tune:
    t = Tune()
    for k, v in kw.items():
        setattr(t, k, int(v))
    return t


class Problem:
    """One loaded fixed-source problem (one mc_problem handle)."""

    def __init__(self, io_dir: str, xs_dir: str | None = None):
        L = lib()
        self._h = ctypes.c_void_p()
        st = L.mc_problem_load_xml(os.fsencode(io_dir), os.fsencode(xs_dir) if xs_dir else None,
                                   ctypes.byref(self._h))
        if st != 0:
            msg = L.mc_last_error(self._h).decode() if self._h else "load failed"
            if self._h:
                L.mc_problem_free(self._h)
                self._h = ctypes.c_void_p()
            raise (InputError if st == 1 else McError)(st, msg)
        n = ctypes.c_uint32()
        L.mc_tally_count(self._h, ctypes.byref(n))
        self.n_estimators = n.value
        self.names = []
        self.sizes = []
        for e in range(self.n_estimators):
            buf = ctypes.create_string_buffer(256)
            L.mc_estimator_name(self._h, e, buf, 256)
            self.names.append(buf.value.decode())
            sz = ctypes.c_uint64()
            L.mc_tally_size(self._h, e, ctypes.byref(sz))
            self.sizes.append(sz.value)
        ns = ctypes.c_uint64()
        L.mc_nsample(self._h, ctypes.byref(ns))
        self.nsample = ns.value

    def _check(self, st: int):
        if st != 0:
            raise McError(st, lib().mc_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().mc_problem_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, n: int | None = None, first: int = 0, seed: int = DEFAULT_SEED, mode: str = "replay",
            tune: Tune | None = None, **tune_kw) -> dict:
        if n is None:
            n = self.nsample
        if tune is None and tune_kw:
            tune = make_tune(**tune_kw)
        self._check(lib().mc_run(self._h, first, n, seed, MODES[mode],
                                 ctypes.byref(tune) if tune is not None else None))
        return self.counters()

    def reset(self):
        self._check(lib().mc_reset_tallies(self._h))

    def upload(self):
        """Re-copy the problem tables host -> device (pinned host copy)."""
        self._check(lib().mc_problem_upload(self._h))

    def table_bytes(self) -> int:
        v = ctypes.c_uint64()
        self._check(lib().mc_problem_table_bytes(self._h, ctypes.byref(v)))
        return v.value

    def counters(self) -> dict:
        c = Counters()
        self._check(lib().mc_counters_read(self._h, ctypes.byref(c)))
        return c.as_dict()

    def tally(self, e: int):
        nb = self.sizes[e]
        m, s, su, sq = (np.zeros(max(nb, 1)) for _ in range(4))
        self._check(lib().mc_tally_read(self._h, e, m.ctypes.data, s.ctypes.data, su.ctypes.data,
                                        sq.ctypes.data, max(nb, 1)))
        return m[:nb], s[:nb], su[:nb], sq[:nb]

    def all_tallies(self):
        parts = [self.tally(e) for e in range(self.n_estimators)]
        if not parts:
            return (np.zeros(0),) * 4
        return tuple(np.concatenate([p[k] for p in parts]) for k in range(4))

    def exact_sums(self) -> np.ndarray:
        """Exact per-bin sums of the FP64 runs since the last reset
        (mc_exact_sums_read): int64 limbs shaped [bins, 2, EXACT_LIMBS]
        (sum of history totals, sum of their squares)."""
        nb = int(sum(self.sizes))
        out = np.zeros((max(nb, 1), 2, EXACT_LIMBS), np.int64)
        self._check(lib().mc_exact_sums_read(self._h, out.ctypes.data, out.size))
        return out[:nb]

    def digests(self, n: int) -> np.ndarray:
        d = np.zeros(n, np.uint64)
        self._check(lib().mc_digests_read(self._h, d.ctypes.data, n))
        return d

    def histories_run(self) -> int:
        v = ctypes.c_uint64()
        self._check(lib().mc_histories_run(self._h, ctypes.byref(v)))
        return v.value

    def save_state(self, path: str):
        """Checkpoint the accumulated tallies (include/mcgpu.h, mc_state_save)."""
        self._check(lib().mc_state_save(self._h, path.encode()))

    def load_state(self, path: str):
        """Resume from a checkpoint of the same problem (mc_state_load)."""
        self._check(lib().mc_state_load(self._h, path.encode()))

    def report(self, path: str):
        self._check(lib().mc_report(self._h, os.fsencode(path)))

    # ---- derivatives (one-group multigroup problems) ----
    def lr_params(self) -> np.ndarray:
        """The materials' one-group (Sigma_s, Sigma_a), interleaved."""
        out = np.zeros(128)
        self._check(lib().mc_lr_params(self._h, out.ctypes.data, 128))
        return out[: 2 * self._n_materials()]

    def _n_materials(self) -> int:
        out = np.zeros(128)
        lib().mc_lr_params(self._h, out.ctypes.data, 128)
        nz = np.nonzero(out)[0]
        return (int(nz[-1]) // 2 + 1) if nz.size else 0

    def forward(self, params, n: int, seed: int = DEFAULT_SEED):
        """(mean, sigma) of every tally bin at the given parameters."""
        p = np.ascontiguousarray(params, np.float64)
        nb = int(sum(self.sizes))
        m = np.zeros(max(nb, 1))
        s = np.zeros(max(nb, 1))
        self._check(lib().mc_forward(self._h, p.ctypes.data, n, seed, m.ctypes.data, s.ctypes.data))
        return m[:nb], s[:nb]

    def backward(self, params, n: int, seed: int = DEFAULT_SEED):
        """(d tally / d params, sigma), shaped [bins, params]."""
        p = np.ascontiguousarray(params, np.float64)
        nb = int(sum(self.sizes))
        K = p.size
        d = np.zeros(max(nb * K, 1))
        s = np.zeros(max(nb * K, 1))
        self._check(lib().mc_backward(self._h, p.ctypes.data, n, seed, d.ctypes.data, s.ctypes.data))
        return d[: nb * K].reshape(nb, K), s[: nb * K].reshape(nb, K)

    def backward_density(self, params, n: int, seed: int = DEFAULT_SEED):
        """(d tally / d params, sigma, rho d tally / d rho, sigma), shaped
        [bins, params] and [bins, materials], from one run."""
        p = np.ascontiguousarray(params, np.float64)
        nb = int(sum(self.sizes))
        K = p.size
        M = K // 2
        d = np.zeros(max(nb * K, 1))
        s = np.zeros(max(nb * K, 1))
        r = np.zeros(max(nb * M, 1))
        rs = np.zeros(max(nb * M, 1))
        self._check(lib().mc_backward_density(self._h, p.ctypes.data, n, seed, d.ctypes.data, s.ctypes.data,
                                              r.ctypes.data, rs.ctypes.data))
        return (d[: nb * K].reshape(nb, K), s[: nb * K].reshape(nb, K),
                r[: nb * M].reshape(nb, M), rs[: nb * M].reshape(nb, M))

    def autotune(self, sample: int = 0, seed: int = DEFAULT_SEED) -> dict:
        """Pick and keep the event engine's fastest launch shape (sample 0:
        the library's default, 8 histories per thread of the largest shape)."""
        t = Tune()
        self._check(lib().mc_autotune(self._h, sample, seed, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}


def batch_problem_seed(seed: int, i: int) -> int:
    """Seed of problem i inside a batch run with `seed` (include/mcgpu.h)."""
    return (seed + 0x9E3779B97F4A7C15 * (i + 1)) & 0xFFFFFFFFFFFFFFFF


class Batch:
    """Many loaded problems run together in one persistent launch."""

    def __init__(self, problems, histories):
        L = lib()
        self.problems = list(problems)
        arr = (ctypes.c_void_p * len(self.problems))(*[p._h.value for p in self.problems])
        hist = (ctypes.c_uint64 * len(self.problems))(*[int(h) for h in histories])
        self.histories = [int(h) for h in histories]
        self._h = ctypes.c_void_p()
        st = L.mc_batch_create(arr, len(self.problems), hist, ctypes.byref(self._h))
        if st != 0:
            msg = L.mc_batch_last_error(self._h).decode() if self._h else "batch create failed"
            self.close()
            raise McError(st, msg)

    def _check(self, st):
        if st != 0:
            raise McError(st, lib().mc_batch_last_error(self._h).decode())

    def run(self, seed: int = DEFAULT_SEED, tune: Tune | None = None, **tune_kw) -> dict:
        if tune is None and tune_kw:
            tune = make_tune(**tune_kw)
        self._check(lib().mc_batch_run(self._h, seed, ctypes.byref(tune) if tune is not None else None))
        return self.counters()

    def counters(self) -> dict:
        c = Counters()
        self._check(lib().mc_batch_counters(self._h, ctypes.byref(c)))
        return c.as_dict()

    def autotune(self, seed: int = DEFAULT_SEED, fraction: float = 0.05) -> dict:
        t = Tune()
        self._check(lib().mc_batch_autotune(self._h, seed, fraction, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def upload(self):
        """Every problem's tables again from pinned host memory, one wait."""
        self._check(lib().mc_batch_upload(self._h))

    def reset(self):
        """Every problem's tallies zeroed, one wait."""
        self._check(lib().mc_batch_reset(self._h))

    def tallies(self):
        """(mean, sigma, sum, sumsq) of every problem's bins, problem after
        problem, in one read-back (mc_batch_tally_read)."""
        total = int(sum(sum(p.sizes) for p in self.problems))
        out = [np.zeros(max(total, 1)) for _ in range(4)]
        self._check(lib().mc_batch_tally_read(self._h, *[a.ctypes.data for a in out], max(total, 1)))
        return tuple(a[:total] for a in out)

    def close(self):
        if getattr(self, "_h", None):
            lib().mc_batch_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Tally:
    """Estimator.h:257-270 (the fields a caller reads after start())."""
    mean: float
    uncer: float


class Estimator:
    def __init__(self, prob: Problem, index: int):
        self._p = prob
        self._i = index
        self.name = prob.names[index]

    def tally(self, i: int) -> Tally:
        m, s, _, _ = self._p.tally(self._i)
        return Tally(float(m[i]), float(s[i]))

    def tally_size(self) -> int:
        return self._p.sizes[self._i]


class Simulator:
    """The reference's Simulator for the fixed-source path, on the GPU."""

    def __init__(self, io_dir: str, xs_dir: str | None = None, mode: str = "replay",
                 seed: int = DEFAULT_SEED):
        self._p = Problem(io_dir.rstrip("/") or ".", xs_dir)
        self.mode = mode
        self.seed = seed
        self.Nsample = self._p.nsample
        self.Ncycle, self.Npassive = 1, 0
        self.Ntrack = 0
        self.Estimators = [Estimator(self._p, i) for i in range(self._p.n_estimators)]

    def start(self):
        c = self._p.run(self.Nsample, 0, self.seed, self.mode)
        self.Ntrack = int(c["flights"])

    def report(self, io_dir: str):
        self._p.report(os.path.join(io_dir, "output.json"))
