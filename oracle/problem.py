"""CPU oracle front end: input.xml -> flat arrays -> mc_oracle.c.

TEST INFRASTRUCTURE.  This module is the oracle's own reader of the
reference's XML schema (MC-old src/simulator/setup.cpp:30-1066).  It is
independent of the product's C++ reader on purpose: the two are compared on
the same inputs.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py may import it.

Schema extensions beyond the reference:
  <population_control><weight_roulette wr=".." ws=".."/>   (simulator.h:90-91)
  <multigroup groups="G"/> plus <material><multigroup total=".." scatter=".."/>
  <isotropic_hemisphere name=".." datatype="point"/>  (cosine to +x ~ U(0,1))
  <point ... group="g"/>  (multigroup source group, 0-based)
  <filter type="group"/>  (one bin per group)
"""
from __future__ import annotations

import ctypes
import math
import os
import re
import subprocess
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# MC_ORACLE_LIB names another build of the same source (the sanitizer build)
LIB_PATH = os.environ.get("MC_ORACLE_LIB") or os.path.join(HERE, "_build", "liboracle.so")

# enums of mc_oracle.h
PX, PY, PZ, PLANE, SPHERE, CYLX, CYLY, CYLZ = range(8)
K_TL, K_C, K_NEUTRON = range(3)
S_FLUX, S_ABSORPTION, S_SCATTER, S_CAPTURE, S_TOTAL = range(5)
F_SURFACE, F_CELL, F_ENERGY, F_TIME, F_GROUP = range(5)
D_DELTA, D_ISO, D_XYZ, D_HEMI_X = range(4)
E_DELTA, E_UNIFORM = range(2)
NUC_TABLE, NUC_CONST = range(2)
N_COUNTERS = 10
COUNTER_NAMES = ["flights", "collisions", "crossings", "tally_updates", "particles",
                 "splits", "xs_evals", "freegas_iters", "nuc_lookups", "combs"]

FLT_MAX = float(np.finfo(np.float32).max)


class InputError(ValueError):
    pass


def build(verbose: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, no GPU)."""
    cmd = ["make", "-s", "-C", HERE, "lib"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        d = ctypes.c_double
        L.orc_run.restype = ctypes.c_int
        L.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p]
        L.orc_n_bins.restype = ctypes.c_int64
        L.orc_n_bins.argtypes = [ctypes.c_void_p]
        L.orc_finalize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                   ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_binary_search.restype = ctypes.c_int
        L.orc_binary_search.argtypes = [d, ctypes.c_void_p, ctypes.c_int]
        for name in ("orc_geometry_quad",):
            getattr(L, name).restype = d
            getattr(L, name).argtypes = [d, d, d]
        L.orc_interpolate.restype = d
        L.orc_interpolate.argtypes = [d, d, d, d, d]
        for name in ("orc_log_", "orc_exp_", "orc_sin_", "orc_cos_",
                     "orc_speed_from_energy", "orc_energy_from_speed"):
            getattr(L, name).restype = d
            getattr(L, name).argtypes = [d]
        L.orc_surface_distance.restype = d
        L.orc_surface_distance.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_surface_eval.restype = d
        L.orc_surface_eval.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_surface_reflect.restype = None
        L.orc_surface_reflect.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.orc_philox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_lcg_skip.restype = ctypes.c_uint64
        L.orc_lcg_skip.argtypes = [ctypes.c_uint64, ctypes.c_int64]
        L.orc_lcg_next.restype = d
        L.orc_lcg_next.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
        _lib = L
    return _lib


def olog(x: float) -> float:
    return lib().orc_log_(x)


def oexp(x: float) -> float:
    return lib().orc_exp_(x)


# --------------------------------------------------------------------------
# the C struct mirror
# --------------------------------------------------------------------------
_P = ctypes.c_void_p
_FIELDS = [
    ("n_surf", ctypes.c_int32), ("surf_type", _P), ("surf_bc", _P), ("surf_coef", _P),
    ("n_cell", ctypes.c_int32), ("cell_imp", _P), ("cell_mat", _P), ("cell_surf_off", _P),
    ("cell_surf", _P), ("cell_sense", _P), ("cell_tl_off", _P), ("cell_tl", _P),
    ("cell_c_off", _P), ("cell_c", _P), ("surf_est_off", _P), ("surf_est", _P),
    ("n_mat", ctypes.c_int32), ("mat_off", _P), ("mat_nuc", _P), ("mat_dens", _P),
    ("n_nuc", ctypes.c_int32), ("nuc_kind", _P), ("nuc_A", _P), ("nuc_const", _P),
    ("nuc_off", _P), ("nuc_len", _P), ("xs_E", _P), ("xs_S", _P), ("xs_C", _P), ("xs_T", _P),
    ("mg_groups", ctypes.c_int32), ("mg_total", _P), ("mg_scatter", _P), ("mg_scat_tot", _P),
    ("mg_capture", _P),
    ("n_est", ctypes.c_int32), ("est_score_off", _P), ("score_kind", _P), ("score_kernel", _P),
    ("est_filt_off", _P), ("filt_kind", _P), ("filt_size", _P), ("filt_grid_off", _P),
    ("filt_grid_len", _P), ("filt_grid", _P), ("est_factor", _P), ("est_factor_off", _P),
    ("est_bin_off", _P),
    ("n_src", ctypes.c_int32), ("src_pos", _P), ("src_cell", _P), ("src_dir_kind", _P),
    ("src_dir_par", _P), ("src_e_kind", _P), ("src_e_par", _P), ("src_group", _P), ("src_cdf", _P),
    ("wr", ctypes.c_double), ("ws", ctypes.c_double),
    ("comb_bank_max", ctypes.c_int32), ("comb_teeth", ctypes.c_int32),
]


class OrcProblemC(ctypes.Structure):
    _fields_ = _FIELDS


_DT = {"i32": np.int32, "i64": np.int64, "f64": np.float64}
_ARRAY_TYPES = {
    "surf_type": "i32", "surf_bc": "i32", "surf_coef": "f64", "cell_imp": "f64", "cell_mat": "i32",
    "cell_surf_off": "i32", "cell_surf": "i32", "cell_sense": "i32", "cell_tl_off": "i32",
    "cell_tl": "i32", "cell_c_off": "i32", "cell_c": "i32", "surf_est_off": "i32",
    "surf_est": "i32", "mat_off": "i32", "mat_nuc": "i32", "mat_dens": "f64", "nuc_kind": "i32",
    "nuc_A": "f64", "nuc_const": "f64", "nuc_off": "i64", "nuc_len": "i32", "xs_E": "f64",
    "xs_S": "f64", "xs_C": "f64", "xs_T": "f64", "mg_total": "f64", "mg_scatter": "f64",
    "mg_scat_tot": "f64", "mg_capture": "f64", "est_score_off": "i32", "score_kind": "i32",
    "score_kernel": "i32", "est_filt_off": "i32", "filt_kind": "i32", "filt_size": "i32",
    "filt_grid_off": "i64", "filt_grid_len": "i32", "filt_grid": "f64", "est_factor": "f64",
    "est_factor_off": "i32", "est_bin_off": "i64", "src_pos": "f64", "src_cell": "i32",
    "src_dir_kind": "i32", "src_dir_par": "f64", "src_e_kind": "i32", "src_e_par": "f64",
    "src_group": "i32", "src_cdf": "f64",
}


# --------------------------------------------------------------------------
# XML reading with pugixml's lenient attribute semantics
# --------------------------------------------------------------------------
def _read_xml(path: str) -> ET.Element:
    text = open(path, "r", encoding="utf-8", errors="replace").read()
    text = re.sub(r"<\?xml.*?\?>", "", text, flags=re.S)
    return ET.fromstring("<__doc__>" + text + "</__doc__>")


def _num_prefix(s: str) -> str:
    m = re.match(r"\s*[+-]?((\d+\.?\d*)|(\.\d+))([eE][+-]?\d+)?", s)
    return m.group(0) if m else ""


def as_double(node, name, default=0.0) -> float:
    v = node.get(name) if node is not None else None
    if v is None:
        return default
    p = _num_prefix(v)
    if not p:
        low = v.strip().lower()
        if low in ("inf", "+inf", "infinity"):
            return math.inf
        return default
    return float(p)


def as_int(node, name, default=0) -> int:
    v = node.get(name) if node is not None else None
    if v is None:
        return default
    m = re.match(r"\s*([+-]?\d+)", v)
    return int(m.group(1)) if m else default


def _doubles(s: str):
    out = []
    for tok in s.split():
        try:
            out.append(float(tok))
        except ValueError:
            break
    return out


@dataclass
class Problem:
    """Flat problem tables (numpy) plus the ctypes struct that points at them."""
    arrays: dict = field(default_factory=dict)
    scalars: dict = field(default_factory=dict)
    name: str = ""
    nsample: int = 0
    est_names: list = field(default_factory=list)
    est_score_names: list = field(default_factory=list)
    _c: OrcProblemC | None = None

    def c_struct(self) -> OrcProblemC:
        if self._c is None:
            c = OrcProblemC()
            for fname, ftype in _FIELDS:
                if ftype is _P:
                    a = self.arrays.get(fname)
                    if a is None or a.size == 0:
                        a = np.zeros(1, dtype=_DT[_ARRAY_TYPES[fname]])
                        self.arrays[fname] = a
                    setattr(c, fname, a.ctypes.data)
                else:
                    setattr(c, fname, self.scalars[fname])
            self._c = c
        return self._c

    @property
    def n_bins(self) -> int:
        return int(self.arrays["est_bin_off"][-1])

    def est_bins(self, e: int):
        off = self.arrays["est_bin_off"]
        return int(off[e]), int(off[e + 1])


def _offsets(lists):
    off = np.zeros(len(lists) + 1, dtype=np.int32)
    for i, l in enumerate(lists):
        off[i + 1] = off[i] + len(l)
    return off


def _csr(lists):
    off = np.zeros(len(lists) + 1, dtype=np.int32)
    flat = []
    for i, l in enumerate(lists):
        flat.extend(l)
        off[i + 1] = len(flat)
    return off, np.array(flat, dtype=np.int32)


def load(io_dir: str, xs_dir: str | None = None) -> Problem:
    """Read io_dir/input.xml the way Simulator::Simulator does (setup.cpp:30)."""
    if xs_dir is None:
        xs_dir = os.path.join(os.getcwd(), "xs_library")
    doc = _read_xml(os.path.join(io_dir, "input.xml"))
    pb = Problem()
    sim = doc.find("simulation")
    desc = sim.find("description") if sim is not None else None
    pb.name = desc.get("name", "") if desc is not None else ""
    pb.nsample = int(as_double(desc, "samples"))
    if sim is not None and (sim.find("ksearch") is not None or sim.find("tdmc") is not None):
        raise InputError("k-eigenvalue and time-dependent modes are out of scope")
    if doc.find("trmm") is not None:
        raise InputError("TRMM is out of scope")

    wr, ws = 0.001, 1.0
    bank_max = teeth = 0
    ctrl = doc.find("population_control")
    if ctrl is not None:
        comb = ctrl.find("particle_comb")
        if comb is not None:   # setup.cpp:57-67
            bank_max = as_int(comb, "bank_max")
            teeth = as_int(comb, "teeth")
            if bank_max < 1 or teeth < 1:
                raise InputError("particle_comb needs bank_max >= 1 and teeth >= 1")
            if teeth > bank_max:   # the reference's history loop never ends
                raise InputError("particle_comb with teeth > bank_max never empties the bank")
        wrn = ctrl.find("weight_roulette")
        if wrn is not None:
            wr = as_double(wrn, "wr", wr)
            ws = as_double(wrn, "ws", ws)

    mg = doc.find("multigroup")
    G = as_int(mg, "groups") if mg is not None else 0

    # ---- distributions (setup.cpp:174-305) ----
    ddist, pdist = {}, {}
    dnode = doc.find("distributions")
    if dnode is not None:
        pending = list(dnode)
        while pending:
            progressed = False
            rest = []
            for d in pending:
                typ, nm, dt = d.tag, d.get("name", ""), d.get("datatype", "")
                if dt == "double":
                    if nm in ddist:
                        progressed = True
                        continue
                    if typ == "delta":
                        ddist[nm] = (E_DELTA, as_double(d, "val"), 0.0)
                    elif typ == "uniform":
                        a, b = as_double(d, "a"), as_double(d, "b")
                        ddist[nm] = (E_UNIFORM, a, b - a)
                    else:
                        raise InputError(f"unsupported double distribution {typ}")
                    progressed = True
                elif dt == "point":
                    if nm in pdist:
                        progressed = True
                        continue
                    if typ == "delta":
                        pdist[nm] = (D_DELTA, [as_double(d, "x"), as_double(d, "y"), as_double(d, "z")])
                    elif typ == "isotropic":
                        pdist[nm] = (D_ISO, [])
                    elif typ == "isotropic_hemisphere":
                        pdist[nm] = (D_HEMI_X, [])
                    elif typ == "independentXYZ":
                        parts = [d.get("x", ""), d.get("y", ""), d.get("z", "")]
                        if not all(p in ddist for p in parts):
                            rest.append(d)
                            continue
                        par = []
                        for p in parts:
                            k, a, r = ddist[p]
                            par += [float(k), a, r]
                        pdist[nm] = (D_XYZ, par)
                    else:
                        raise InputError(f"unsupported point distribution {typ}")
                    progressed = True
                else:
                    raise InputError(f"unsupported distribution datatype {dt}")
            if not progressed:
                raise InputError("distributions could not be resolved")
            pending = rest

    # ---- nuclides (setup.cpp:310-467) ----
    nuc_names, nuc_kind, nuc_A, nuc_const = [], [], [], []
    nuc_off, nuc_len, xsE, xsS, xsC, xsT = [], [], [], [], [], []
    npts = 0
    nnode = doc.find("nuclides")
    for n in (nnode.findall("nuclide") if nnode is not None else []):
        nuc_names.append(n.get("name", ""))
        if n.get("ZAID") is not None:
            path = os.path.join(xs_dir, n.get("ZAID") + ".txt")
            try:
                toks = open(path).read().split()
            except OSError as e:
                raise InputError(f"cannot read {path}: {e}")
            vals = []
            for t in toks:
                try:
                    vals.append(float(t))
                except ValueError:
                    break
            if len(vals) < 7:
                raise InputError(f"short cross-section file {path}")
            A = vals[0]
            rows = (len(vals) - 7) // 6
            tab = np.array(vals[7:7 + 6 * rows], dtype=np.float64).reshape(rows, 6)
            if np.any(tab[:, 3] != 0.0):
                raise InputError(f"{path}: fissile data (sigma_f != 0) is out of scope")
            nuc_kind.append(NUC_TABLE)
            nuc_A.append(A)
            nuc_const.append(0.0)
            nuc_off.append(npts)
            nuc_len.append(rows)
            npts += rows
            xsE.append(tab[:, 0])
            xsS.append(tab[:, 1])
            xsC.append(tab[:, 2] + tab[:, 3])          # sigma_a = c + f
            xsT.append(tab[:, 1] + tab[:, 2] + tab[:, 3])  # (c2 + c3) + c4
        else:
            cap = None
            for r in list(n):
                if r.get("xs") is None:
                    raise InputError("unknown XS type")
                if r.tag != "capture":
                    raise InputError("user-defined nuclides support capture only")
                cap = as_double(r, "xs")
            nuc_kind.append(NUC_CONST)
            nuc_A.append(as_double(n, "A", FLT_MAX))
            nuc_const.append(0.0 if cap is None else cap)
            nuc_off.append(npts)
            nuc_len.append(0)

    # ---- materials (setup.cpp:474-492) ----
    mat_names, mat_lists = [], []
    mg_total, mg_scatter = [], []
    mnode = doc.find("materials")
    for m in (mnode.findall("material") if mnode is not None else []):
        mat_names.append(m.get("name", ""))
        mgn = m.find("multigroup")
        if G > 0:
            if mgn is None:
                raise InputError("multigroup problem needs <multigroup> data in every material")
            tot = _doubles(mgn.get("total", ""))
            sca = _doubles(mgn.get("scatter", ""))
            if len(tot) != G or len(sca) != G * G:
                raise InputError("multigroup data has the wrong size")
            mg_total.append(tot)
            mg_scatter.append(sca)
            mat_lists.append([])
            continue
        lst = []
        for nn in m.findall("nuclide"):
            nm = nn.get("name", "")
            if nm not in nuc_names:
                raise InputError("unknown nuclide")
            lst.append((nuc_names.index(nm), as_double(nn, "density")))
        mat_lists.append(lst)

    # ---- surfaces (setup.cpp:499-584) ----
    surf_names, stype, sbc, scoef = [], [], [], []
    snode = doc.find("surfaces")
    for s in (list(snode) if snode is not None else []):
        bc = s.get("bc", "transmission")
        bcv = {"transmission": 0, "reflective": 1, "vacuum": -1}.get(bc)
        if bcv is None:
            raise InputError(f"unknown boundary condition {bc}")
        c = [0.0] * 8
        t = s.tag
        if t == "plane_x":
            typ, c[0] = PX, as_double(s, "x")
        elif t == "plane_y":
            typ, c[0] = PY, as_double(s, "y")
        elif t == "plane_z":
            typ, c[0] = PZ, as_double(s, "z")
        elif t == "plane":
            typ = PLANE
            a, b, cc, d = (as_double(s, k) for k in "abcd")
            L = 2.0 / (a * a + b * b + cc * cc)
            c[:7] = [a, b, cc, d, L * a, L * b, L * cc]
        elif t == "sphere":
            typ = SPHERE
            r = as_double(s, "r")
            c[:5] = [as_double(s, "x"), as_double(s, "y"), as_double(s, "z"), r, r * r]
        elif t == "cylinder_x":
            typ = CYLX
            r = as_double(s, "r")
            c[:4] = [as_double(s, "y"), as_double(s, "z"), r, r * r]
        elif t == "cylinder_z":
            typ = CYLZ
            r = as_double(s, "r")
            c[:4] = [as_double(s, "x"), as_double(s, "y"), r, r * r]
        else:
            raise InputError(f"unknown surface type {t}")
        surf_names.append(s.get("name", ""))
        stype.append(typ)
        sbc.append(bcv)
        scoef.append(c)

    # ---- cells (setup.cpp:591-629) ----
    cell_names, cimp, cmat, csurf = [], [], [], []
    cnode = doc.find("cells")
    for c in (cnode.findall("cell") if cnode is not None else []):
        cell_names.append(c.get("name", f"Cell {len(cell_names) + 1}"))
        cimp.append(as_double(c, "importance", 1.0) if c.get("importance") is not None else 1.0)
        if c.get("material") is not None:
            if c.get("material") not in mat_names:
                raise InputError("unknown material in cell")
            cmat.append(mat_names.index(c.get("material")))
        else:
            cmat.append(-1)
        lst = []
        for sn in c.findall("surface"):
            nm = sn.get("name", "")
            if nm not in surf_names:
                raise InputError("unknown surface")
            lst.append((surf_names.index(nm), as_int(sn, "sense")))
        csurf.append(lst)

    # ---- estimators (setup.cpp:637-805) ----
    cell_tl = [[] for _ in cell_names]
    cell_c = [[] for _ in cell_names]
    surf_est = [[] for _ in surf_names]
    e_scores_kind, e_scores_kernel, e_filters, est_names, est_snames = [], [], [], [], []
    enode = doc.find("estimators")
    for e in (enode.findall("estimator") if enode is not None else []):
        ei = len(est_names)
        est_names.append(e.get("name", f"Estimator #{ei + 1}"))
        etype = e.get("type", "TL")
        if etype == "TL":
            kern = K_TL
        elif etype == "C":
            kern = K_C
        else:
            raise InputError("unsupported estimator type")
        if e.get("scores") is None:
            raise InputError("estimator without scores")
        kinds, kernels, snames = [], [], []
        for sname in e.get("scores").split():
            if sname == "flux":
                k = S_FLUX
            elif sname == "absorption":
                k = S_ABSORPTION
            elif sname == "scatter":
                k = S_SCATTER
            elif sname == "capture":
                k = S_CAPTURE
            elif sname == "total":
                k = S_TOTAL
            elif sname == "cross":
                kern = K_NEUTRON        # setup.cpp:688-690 switches the kernel for later scores too
                k = S_FLUX
            else:
                raise InputError(f"unsupported score {sname}")
            kinds.append(k)
            kernels.append(kern)
            snames.append(sname)
        filters = []
        grid = []
        surfs = e.findall("surface")
        cells = e.findall("cell")
        if surfs and cells:
            raise InputError("an estimator is attached to surfaces or to cells, not both")
        for sn in surfs:
            nm = sn.get("name", "")
            if nm not in surf_names:
                raise InputError("unknown surface in estimator")
            si = surf_names.index(nm)
            surf_est[si].append(ei)
            grid.append(float(si))
        for cn in cells:
            nm = cn.get("name", "")
            if nm not in cell_names:
                raise InputError("unknown cell in estimator")
            ci = cell_names.index(nm)
            if etype == "TL":
                cell_tl[ci].append(ei)
            else:
                cell_c[ci].append(ei)
            grid.append(float(ci))
        if surfs:
            filters.append((F_SURFACE, grid, len(grid)))
        elif cells:
            filters.append((F_CELL, grid, len(grid)))
        else:
            raise InputError("estimator needs to be attached somewhere")
        for f in e.findall("filter"):
            ftype = f.get("type", "")
            if ftype == "group":
                if G <= 0:
                    raise InputError("group filter needs a multigroup problem")
                filters.append((F_GROUP, [float(g) for g in range(G + 1)], G))
                continue
            if f.get("grid") is not None:
                fg = _doubles(f.get("grid"))
            elif f.get("grid_linear") is not None:
                a, step, b = (_doubles(f.get("grid_linear")) + [0, 0, 0])[:3]
                fg = [a]
                while fg[-1] < b:
                    fg.append(fg[-1] + step)
                fg.pop()
                fg.append(b)
            elif f.get("grid_lethargy") is not None:
                a, b, N = (_doubles(f.get("grid_lethargy")) + [0, 0, 0])[:3]
                step = olog(b / a) / N
                fg = [0.0]
                while len(fg) != N + 1:
                    fg.append(fg[-1] + step)
                fg.reverse()
                fg = [b * oexp(-v) for v in fg]
            else:
                raise InputError("filter needs a grid")
            if ftype == "energy":
                filters.append((F_ENERGY, fg, len(fg) - 1))
            elif ftype == "time":
                filters.append((F_TIME, fg, len(fg) - 1))
            else:
                raise InputError("unknown filter type")
        e_scores_kind.append(kinds)
        e_scores_kernel.append(kernels)
        e_filters.append(filters)
        est_snames.append(snames)

    # ---- sources (setup.cpp:1020-1066) ----
    src_pos, src_cell, sdk, sdp, sek, sep, sgrp = [], [], [], [], [], [], []
    srcnode = doc.find("sources")
    for s in (list(srcnode) if srcnode is not None else []):
        dk, dpar = D_ISO, []
        ek, ea, er = E_DELTA, 2e6, 0.0
        if s.get("direction") is not None:
            if s.get("direction") not in pdist:
                raise InputError("unknown direction distribution in source")
            dk, dpar = pdist[s.get("direction")]
        if s.get("energy") is not None:
            if s.get("energy") not in ddist:
                raise InputError("unknown energy distribution in source")
            ek, ea, er = ddist[s.get("energy")]
        if s.tag != "point":
            raise InputError(f"unknown source type {s.tag}")
        p = [as_double(s, "x"), as_double(s, "y"), as_double(s, "z")]
        # search_cell at set-up (setup.cpp:1056, general.cpp:26-34)
        found = -1
        for ci, lst in enumerate(csurf):
            ok = True
            for si, sense in lst:
                if _eval_surface(stype[si], scoef[si], p) * sense < 0:
                    ok = False
                    break
            if ok:
                found = ci
                break
        if found < 0:
            raise InputError("source point is in no cell")
        src_pos.append(p)
        src_cell.append(found)
        sdk.append(dk)
        sdp.append((list(dpar) + [0.0] * 9)[:9])
        sek.append(ek)
        sep.append([ea, er])
        sgrp.append(as_int(s, "group", 0))
    if not src_pos:
        raise InputError("no source")
    nsrc = len(src_pos)
    cdf = [0.0] * (nsrc + 1)
    dp = 1.0 / nsrc
    for i in range(1, nsrc + 1):
        cdf[i] = cdf[i - 1] + dp

    # ---- flatten ----
    A = pb.arrays
    A["surf_type"] = np.array(stype, np.int32)
    A["surf_bc"] = np.array(sbc, np.int32)
    A["surf_coef"] = np.array(scoef, np.float64).reshape(-1)
    A["cell_imp"] = np.array(cimp, np.float64)
    A["cell_mat"] = np.array(cmat, np.int32)
    A["cell_surf_off"], A["cell_surf"] = _csr([[s for s, _ in l] for l in csurf])
    A["cell_sense"] = np.array([v for l in csurf for _, v in l], np.int32)
    A["cell_tl_off"], A["cell_tl"] = _csr(cell_tl)
    A["cell_c_off"], A["cell_c"] = _csr(cell_c)
    A["surf_est_off"], A["surf_est"] = _csr(surf_est)
    A["mat_off"], A["mat_nuc"] = _csr([[n for n, _ in l] for l in mat_lists])
    A["mat_dens"] = np.array([d for l in mat_lists for _, d in l], np.float64)
    A["nuc_kind"] = np.array(nuc_kind, np.int32)
    A["nuc_A"] = np.array(nuc_A, np.float64)
    A["nuc_const"] = np.array(nuc_const, np.float64)
    A["nuc_off"] = np.array(nuc_off, np.int64)
    A["nuc_len"] = np.array(nuc_len, np.int32)
    cat = lambda l: np.concatenate(l) if l else np.zeros(0)
    A["xs_E"], A["xs_S"], A["xs_C"], A["xs_T"] = cat(xsE), cat(xsS), cat(xsC), cat(xsT)
    if G > 0:
        tot = np.array(mg_total, np.float64).reshape(-1, G)
        sca = np.array(mg_scatter, np.float64).reshape(-1, G, G)
        stot = np.zeros_like(tot)
        for m in range(tot.shape[0]):
            for g in range(G):
                acc = 0.0
                for g2 in range(G):
                    acc += float(sca[m, g, g2])
                stot[m, g] = acc
        A["mg_total"] = tot.reshape(-1)
        A["mg_scatter"] = sca.reshape(-1)
        A["mg_scat_tot"] = stot.reshape(-1)
        A["mg_capture"] = (tot - stot).reshape(-1)
    A["est_score_off"] = _offsets(e_scores_kind)
    A["score_kind"] = np.array([k for l in e_scores_kind for k in l], np.int32)
    A["score_kernel"] = np.array([k for l in e_scores_kernel for k in l], np.int32)
    A["est_filt_off"] = _offsets(e_filters)
    fk, fs, fgo, fgl, fg, fac, facoff, binoff = [], [], [], [], [], [], [0], [0]
    for ei, filters in enumerate(e_filters):
        for kind, grid, size in filters:
            fk.append(kind)
            fs.append(size)
            fgo.append(len(fg))
            fgl.append(len(grid))
            fg.extend(grid)
        # Estimator::initialize_tallies (Estimator.cpp:280-295)
        factor = 1.0
        f = [factor]
        for kind, grid, size in reversed(filters):
            factor *= size
            f.insert(0, factor)
        fac.extend(f)
        facoff.append(len(fac))
        ntally = len(e_scores_kind[ei])
        for _, _, size in filters:
            ntally *= size
        binoff.append(binoff[-1] + ntally)
    A["filt_kind"] = np.array(fk, np.int32)
    A["filt_size"] = np.array(fs, np.int32)
    A["filt_grid_off"] = np.array(fgo, np.int64)
    A["filt_grid_len"] = np.array(fgl, np.int32)
    A["filt_grid"] = np.array(fg, np.float64)
    A["est_factor"] = np.array(fac, np.float64)
    A["est_factor_off"] = np.array(facoff, np.int32)
    A["est_bin_off"] = np.array(binoff, np.int64)
    A["src_pos"] = np.array(src_pos, np.float64).reshape(-1)
    A["src_cell"] = np.array(src_cell, np.int32)
    A["src_dir_kind"] = np.array(sdk, np.int32)
    A["src_dir_par"] = np.array(sdp, np.float64).reshape(-1)
    A["src_e_kind"] = np.array(sek, np.int32)
    A["src_e_par"] = np.array(sep, np.float64).reshape(-1)
    A["src_group"] = np.array(sgrp, np.int32)
    A["src_cdf"] = np.array(cdf, np.float64)
    pb.scalars = {"n_surf": len(stype), "n_cell": len(cimp), "n_mat": len(mat_lists),
                  "n_nuc": len(nuc_kind), "mg_groups": G, "n_est": len(est_names),
                  "n_src": nsrc, "wr": wr, "ws": ws,
                  "comb_bank_max": bank_max, "comb_teeth": teeth}
    pb.est_names = est_names
    pb.est_score_names = est_snames
    return pb


def _eval_surface(t, c, p):
    """Surface::eval (Geometry.cpp:29-69), used once for the source cell."""
    if t == PX:
        return p[0] - c[0]
    if t == PY:
        return p[1] - c[0]
    if t == PZ:
        return p[2] - c[0]
    if t == PLANE:
        return c[0] * p[0] + c[1] * p[1] + c[2] * p[2] - c[3]
    if t == SPHERE:
        xt, yt, zt = p[0] - c[0], p[1] - c[1], p[2] - c[2]
        return xt * xt + yt * yt + zt * zt - c[4]
    if t == CYLX:
        yt, zt = p[1] - c[0], p[2] - c[1]
        return yt * yt + zt * zt - c[3]
    if t == CYLY:
        xt, zt = p[0] - c[0], p[1] - c[1]
        return xt * xt + zt * zt - c[3]
    xt, yt = p[0] - c[0], p[1] - c[1]
    return xt * xt + yt * yt - c[3]


@dataclass
class RunResult:
    sum: np.ndarray
    sq: np.ndarray
    counters: np.ndarray
    digest: np.ndarray | None
    hist: np.ndarray | None
    status: int
    nsample: int

    def finalize(self):
        nb = self.sum.size
        mean = np.zeros(nb)
        unc = np.zeros(nb)
        if nb:
            lib().orc_finalize(self.sum.ctypes.data, self.sq.ctypes.data, nb, self.nsample,
                               mean.ctypes.data, unc.ctypes.data)
        return mean, unc


def run(pb: Problem, n: int | None = None, seed: int = 0x4D43, first: int = 0,
        digests: bool = False, hist: bool = False) -> RunResult:
    """Run histories [first, first+n) through the C oracle."""
    if n is None:
        n = pb.nsample
    nb = pb.n_bins
    s = np.zeros(max(nb, 1))
    q = np.zeros(max(nb, 1))
    cnt = np.zeros(N_COUNTERS, np.uint64)
    dg = np.zeros(n, np.uint64) if digests else None
    hh = np.zeros((n, max(nb, 1))) if hist else None
    st = lib().orc_run(ctypes.byref(pb.c_struct()), first, n, seed, s.ctypes.data, q.ctypes.data,
                       cnt.ctypes.data, dg.ctypes.data if digests else None,
                       hh.ctypes.data if hist else None)
    return RunResult(s[:nb], q[:nb], cnt, dg, hh[:, :nb] if hist else None, st, n)
