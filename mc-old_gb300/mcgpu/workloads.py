"""Synthetic fixed-source workloads written in the reference's input format.

Each writer produces a directory holding ``input.xml`` (the schema read by
MC-old's Simulator, src/simulator/setup.cpp:30-1066) and, for
continuous-energy problems, an ``xs_library/`` of 6-column tables
(xs_library/README.txt:1-7: energy, sigma_s, sigma_c, sigma_f, nu, nu_d).
Random parameters come from ``numpy.random.Generator(PCG64(1000 + k))`` where
``k`` is the workload's number.  Only uniform draws and IEEE arithmetic
(+, -, *, /, sqrt) touch the written numbers; logarithms and exponentials go
through Python's ``decimal`` module, which rounds correctly, so every writer
produces the same bytes on every machine (libm and numpy's exp/log differ in
the last bit between x86-64 and aarch64).

Workloads (sizes are the defaults; all can be shrunk for tests):
  slab_1g            20 cm 1-group slab, sigma_t = 1, c = 0.5, inward
                     hemisphere plane source at x = 0+, transmission,
                     reflection, absorption and a 100-bin track-length flux.
  ce_sphere          three-shell continuous-energy shield (water-like,
                     graphite, borated graphite) with a 2 MeV isotropic point
                     source, 20,000-point log-uniform synthetic tables for
                     H1, O16, C, B10, B11, leakage current, a 50-bin lethargy
                     spectrum in the outer shell and per-shell flux.
  mg_deep_slab       100 cm, 5 regions, 30 groups, downscatter P0 matrix,
                     weight roulette 0.25 -> 1.0, importance 2^r.
  mg_layered_slab    16 x 1 cm single-group regions (the differentiation
                     workload).
  batch_shields      4096 independent multigroup slab or sphere shields of
                     uneven size (1-8 regions, 1 or 8 groups, 1-50 mean free
                     paths, 10^3-10^6 histories each, log-uniform).
"""
from __future__ import annotations

import decimal
import math
import os

import numpy as np

FMT = "%.17g"


def _rng(k: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(1000 + k))


def log_uniform_grid(lo: float, hi: float, n: int) -> np.ndarray:
    """n points, log-uniform from lo to hi, each exp(ln lo + i*step) rounded
    once from 40-digit decimal arithmetic (identical on every platform)."""
    ctx = decimal.Context(prec=40)
    a = ctx.ln(decimal.Decimal(repr(lo)))
    b = ctx.ln(decimal.Decimal(repr(hi)))
    step = ctx.divide(ctx.subtract(b, a), decimal.Decimal(n - 1))
    out = np.empty(n)
    for i in range(n):
        out[i] = float(ctx.exp(ctx.add(a, ctx.multiply(step, decimal.Decimal(i)))))
    out[0], out[-1] = lo, hi
    return out


def dirichlet1(rng: np.random.Generator, k: int) -> np.ndarray:
    """Dirichlet(1, ..., 1) on k components as the spacings of k-1 sorted
    uniforms (uniform on the simplex; needs no logarithm)."""
    if k == 1:
        return np.ones(1)
    u = np.sort(rng.uniform(0.0, 1.0, size=k - 1))
    edges = np.concatenate([[0.0], u, [1.0]])
    return np.diff(edges)


def write_xs_table(path: str, A: float, E, sig_s, sig_c) -> None:
    """Write one nuclide in the 6-column xs_library format."""
    E = np.asarray(E, np.float64)
    sig_s = np.broadcast_to(np.asarray(sig_s, np.float64), E.shape)
    sig_c = np.broadcast_to(np.asarray(sig_c, np.float64), E.shape)
    with open(path, "w") as f:
        f.write(FMT % A + "\n")
        for _ in range(3):
            f.write("0 0\n")
        z = np.zeros_like(E)
        tab = np.stack([E, sig_s, sig_c, z, z, z], axis=1)
        np.savetxt(f, tab, fmt=FMT, delimiter=" ")


def _xml_header(name: str, samples: int) -> str:
    return ("<?xml version = '1.0' encoding = 'UTF-8'?>\n"
            f"<simulation>\n    <description name=\"{name}\" samples=\"{samples:d}\"/>\n"
            "</simulation>\n")


def _fmt(v: float) -> str:
    return FMT % v


def slab_1g(out_dir: str, samples: int = 1_000_000, thickness: float = 20.0,
            sig_t: float = 1.0, sig_s: float = 0.5, n_flux_bins: int = 100,
            big_A: float = 1e30) -> str:
    """1-group homogeneous slab with an inward plane source at x = 0+.

    One group is written as a 2-point table with constant cross sections and
    a nuclide mass of 1e30 so that the reference's free-gas elastic scatter
    (Reaction.cpp:27-118) reduces to isotropic scattering in the lab frame.
    The 100-bin flux uses 100 cells of 0.2 cm; leakage uses transmission
    planes and importance-0 graveyard cells, the way the reference's examples
    score leakage (examples/slab_analytic/input.xml).
    """
    os.makedirs(os.path.join(out_dir, "xs_library"), exist_ok=True)
    write_xs_table(os.path.join(out_dir, "xs_library", "900001.txt"), big_A,
                   [1e-5, 2e7], [sig_s, sig_s], [sig_t - sig_s, sig_t - sig_s])
    w = n_flux_bins
    dx = thickness / w
    xs = [_fmt(i * dx) if i < w else _fmt(thickness) for i in range(w + 1)]
    s = [_xml_header("slab_1g", samples)]
    s.append("<nuclides>\n    <nuclide name=\"one\" ZAID=\"900001\"/>\n</nuclides>\n")
    s.append("<materials>\n    <material name=\"m\">\n        <nuclide name=\"one\" density=\"1.0\"/>\n"
             "    </material>\n</materials>\n")
    s.append("<surfaces>\n")
    for i, x in enumerate(xs):
        s.append(f"    <plane_x name=\"p{i}\" x=\"{x}\"/>\n")
    s.append("</surfaces>\n<cells>\n")
    for i in range(w):
        s.append(f"    <cell name=\"c{i}\" material=\"m\">\n"
                 f"        <surface name=\"p{i}\" sense=\"+1\"/>\n"
                 f"        <surface name=\"p{i + 1}\" sense=\"-1\"/>\n    </cell>\n")
    s.append(f"    <cell name=\"left\" importance=\"0.0\">\n        <surface name=\"p0\" sense=\"-1\"/>\n    </cell>\n")
    s.append(f"    <cell name=\"right\" importance=\"0.0\">\n        <surface name=\"p{w}\" sense=\"+1\"/>\n    </cell>\n")
    s.append("</cells>\n")
    s.append("<distributions>\n    <isotropic_hemisphere name=\"inward\" datatype=\"point\"/>\n</distributions>\n")
    s.append("<sources>\n    <point x=\"1e-9\" y=\"0.0\" z=\"0.0\" direction=\"inward\"/>\n</sources>\n")
    s.append("<estimators>\n")
    s.append(f"    <estimator name=\"transmission\" scores=\"cross\">\n        <surface name=\"p{w}\"/>\n    </estimator>\n")
    s.append("    <estimator name=\"reflection\" scores=\"cross\">\n        <surface name=\"p0\"/>\n    </estimator>\n")
    s.append("    <estimator name=\"slab\" scores=\"flux absorption\">\n")
    for i in range(w):
        s.append(f"        <cell name=\"c{i}\"/>\n")
    s.append("    </estimator>\n</estimators>\n")
    with open(os.path.join(out_dir, "input.xml"), "w") as f:
        f.write("".join(s))
    return out_dir


CE_NUCLIDES = [  # name, ZAID, A
    ("H1", "001001", 1.0),
    ("O16", "008016", 16.0),
    ("C", "006000", 12.0),
    ("B10", "005010", 10.0),
    ("B11", "005011", 11.0),
]


def ce_tables(n_points: int = 20_000, k: int = 2):
    """Synthetic pointwise cross sections: sigma_s = s0/(1+E/Ec),
    sigma_c = c0*sqrt(0.0253/E) on a log-uniform grid 1e-5 eV .. 20 MeV."""
    rng = _rng(k)
    E = log_uniform_grid(1e-5, 2e7, n_points)
    out = {}
    for name, zaid, A in CE_NUCLIDES:
        s0 = rng.uniform(2.0, 20.0)
        Ec = rng.uniform(0.1e6, 5.0e6)
        c0 = 3840.0 if name == "B10" else rng.uniform(0.1, 1.0)
        if name == "B10":
            rng.uniform(0.1, 1.0)   # keep the stream aligned across nuclides
        out[name] = (zaid, A, E, s0 / (1.0 + E / Ec), c0 * np.sqrt(0.0253 / E))
    return out


def ce_sphere(out_dir: str, samples: int = 10_000_000, n_points: int = 20_000,
              radii=(30.0, 60.0, 70.0), n_spectrum: int = 50) -> str:
    """Continuous-energy three-shell spherical shield, 2 MeV point source."""
    os.makedirs(os.path.join(out_dir, "xs_library"), exist_ok=True)
    for name, (zaid, A, E, ss, sc) in ce_tables(n_points).items():
        write_xs_table(os.path.join(out_dir, "xs_library", zaid + ".txt"), A, E, ss, sc)
    r1, r2, r3 = radii
    s = [_xml_header("ce_sphere", samples)]
    s.append("<nuclides>\n")
    for name, zaid, _ in CE_NUCLIDES:
        s.append(f"    <nuclide name=\"{name}\" ZAID=\"{zaid}\"/>\n")
    s.append("</nuclides>\n<materials>\n"
             "    <material name=\"water\">\n        <nuclide name=\"H1\" density=\"0.0667\"/>\n"
             "        <nuclide name=\"O16\" density=\"0.0334\"/>\n    </material>\n"
             "    <material name=\"graphite\">\n        <nuclide name=\"C\" density=\"0.08\"/>\n    </material>\n"
             "    <material name=\"borated\">\n        <nuclide name=\"B10\" density=\"0.002\"/>\n"
             "        <nuclide name=\"B11\" density=\"0.008\"/>\n        <nuclide name=\"C\" density=\"0.07\"/>\n"
             "    </material>\n</materials>\n")
    s.append("<surfaces>\n"
             f"    <sphere name=\"s1\" x=\"0\" y=\"0\" z=\"0\" r=\"{_fmt(r1)}\"/>\n"
             f"    <sphere name=\"s2\" x=\"0\" y=\"0\" z=\"0\" r=\"{_fmt(r2)}\"/>\n"
             f"    <sphere name=\"s3\" x=\"0\" y=\"0\" z=\"0\" r=\"{_fmt(r3)}\"/>\n</surfaces>\n")
    s.append("<cells>\n"
             "    <cell name=\"core\" material=\"water\">\n        <surface name=\"s1\" sense=\"-1\"/>\n    </cell>\n"
             "    <cell name=\"mid\" material=\"graphite\">\n        <surface name=\"s1\" sense=\"+1\"/>\n"
             "        <surface name=\"s2\" sense=\"-1\"/>\n    </cell>\n"
             "    <cell name=\"outer\" material=\"borated\">\n        <surface name=\"s2\" sense=\"+1\"/>\n"
             "        <surface name=\"s3\" sense=\"-1\"/>\n    </cell>\n"
             "    <cell name=\"graveyard\" importance=\"0.0\">\n        <surface name=\"s3\" sense=\"+1\"/>\n    </cell>\n"
             "</cells>\n")
    s.append("<distributions>\n    <delta name=\"E0\" datatype=\"double\" val=\"2e6\"/>\n"
             "    <isotropic name=\"iso\" datatype=\"point\"/>\n</distributions>\n")
    s.append("<sources>\n    <point x=\"0\" y=\"0\" z=\"0\" direction=\"iso\" energy=\"E0\"/>\n</sources>\n")
    s.append("<estimators>\n"
             "    <estimator name=\"leakage\" scores=\"cross\">\n        <surface name=\"s3\"/>\n    </estimator>\n"
             "    <estimator name=\"outer_spectrum\" scores=\"flux\">\n        <cell name=\"outer\"/>\n"
             f"        <filter type=\"energy\" grid_lethargy=\"1e-5 2e7 {n_spectrum}\"/>\n    </estimator>\n"
             "    <estimator name=\"shell_flux\" scores=\"flux\">\n        <cell name=\"core\"/>\n"
             "        <cell name=\"mid\"/>\n        <cell name=\"outer\"/>\n    </estimator>\n"
             "</estimators>\n")
    with open(os.path.join(out_dir, "input.xml"), "w") as f:
        f.write("".join(s))
    return out_dir


def mg_slab_data(n_regions: int, G: int, k: int, c_lo=0.5, c_hi=0.95, st_lo=0.2, st_hi=2.0,
                 downscatter_only: bool = True, rng: np.random.Generator | None = None):
    """Per-region multigroup data: sigma_t[g] ~ U[st_lo, st_hi], scatter
    ratio c_g ~ U[c_lo, c_hi] split over g' >= g by Dirichlet(1).  The last
    group has no lower group, so self-scatter g' = g is always included."""
    rng = rng or _rng(k)
    tot = rng.uniform(st_lo, st_hi, size=(n_regions, G))
    sca = np.zeros((n_regions, G, G))
    for r in range(n_regions):
        for g in range(G):
            c = rng.uniform(c_lo, c_hi)
            lo = g if downscatter_only else 0
            frac = dirichlet1(rng, G - lo)
            sca[r, g, lo:] = c * tot[r, g] * frac
    return tot, sca


def _mg_slab_xml(out_dir, name, samples, widths, tot, sca, imps, estimators, wr=None, ws=None,
                 source_dir="inward", group=0):
    R, G = tot.shape
    x = [0.0]
    for wdt in widths:
        x.append(x[-1] + wdt)
    s = [_xml_header(name, samples)]
    if wr is not None:
        s.append(f"<population_control>\n    <weight_roulette wr=\"{_fmt(wr)}\" ws=\"{_fmt(ws)}\"/>\n"
                 "</population_control>\n")
    s.append(f"<multigroup groups=\"{G}\"/>\n<materials>\n")
    for r in range(R):
        s.append(f"    <material name=\"m{r}\">\n        <multigroup total=\""
                 + " ".join(_fmt(v) for v in tot[r]) + "\"\n            scatter=\""
                 + " ".join(_fmt(v) for v in sca[r].reshape(-1)) + "\"/>\n    </material>\n")
    s.append("</materials>\n<surfaces>\n")
    for i, xi in enumerate(x):
        s.append(f"    <plane_x name=\"p{i}\" x=\"{_fmt(xi)}\"/>\n")
    s.append("</surfaces>\n<cells>\n")
    for r in range(R):
        s.append(f"    <cell name=\"c{r}\" material=\"m{r}\" importance=\"{_fmt(imps[r])}\">\n"
                 f"        <surface name=\"p{r}\" sense=\"+1\"/>\n"
                 f"        <surface name=\"p{r + 1}\" sense=\"-1\"/>\n    </cell>\n")
    s.append("    <cell name=\"left\" importance=\"0.0\">\n        <surface name=\"p0\" sense=\"-1\"/>\n    </cell>\n")
    s.append(f"    <cell name=\"right\" importance=\"0.0\">\n        <surface name=\"p{R}\" sense=\"+1\"/>\n    </cell>\n")
    s.append("</cells>\n<distributions>\n    <isotropic_hemisphere name=\"inward\" datatype=\"point\"/>\n"
             "</distributions>\n")
    s.append(f"<sources>\n    <point x=\"1e-9\" y=\"0.0\" z=\"0.0\" direction=\"{source_dir}\" group=\"{group}\"/>\n</sources>\n")
    s.append("<estimators>\n" + estimators.replace("@R", str(R)) + "</estimators>\n")
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "input.xml"), "w") as f:
        f.write("".join(s))
    return out_dir


def mg_deep_slab(out_dir: str, samples: int = 100_000_000, n_regions: int = 5, G: int = 30,
                 thickness: float = 100.0) -> str:
    """Deep-penetration multigroup slab with weight roulette and importance
    doubling per region; 30-group transmitted current at x = 100."""
    tot, sca = mg_slab_data(n_regions, G, k=3)
    est = ("    <estimator name=\"transmitted\" scores=\"cross\">\n        <surface name=\"p@R\"/>\n"
           "        <filter type=\"group\"/>\n    </estimator>\n"
           "    <estimator name=\"reflected\" scores=\"cross\">\n        <surface name=\"p0\"/>\n"
           "    </estimator>\n")
    return _mg_slab_xml(out_dir, "mg_deep_slab", samples, [thickness / n_regions] * n_regions,
                        tot, sca, [2.0 ** r for r in range(n_regions)], est, wr=0.25, ws=1.0)


def mg_layered_slab(out_dir: str, samples: int = 10_000_000, n_regions: int = 16,
                    tot=None, c=None, detectors=False) -> str:
    """16 x 1 cm one-group layered slab (the differentiation workload);
    transmitted current at the far face.  detectors="reflected" adds the
    reflected current at x = 0; detectors=True adds it and the current
    through every interface (one bin per plane).  With sigma_t ~ U[0.5, 2]
    the slab is ~22 mean free paths thick and its transmission (~5e-9) is
    far below what 1e7 histories resolve, while these currents are
    resolved."""
    rng = _rng(5)
    if tot is None:
        tot = rng.uniform(0.5, 2.0, size=n_regions)
    if c is None:
        c = rng.uniform(0.3, 0.95, size=n_regions)
    tot = np.asarray(tot, np.float64).reshape(n_regions, 1)
    sca = (np.asarray(c, np.float64).reshape(n_regions, 1) * tot).reshape(n_regions, 1, 1)
    est = ("    <estimator name=\"transmitted\" scores=\"cross\">\n        <surface name=\"p@R\"/>\n"
           "    </estimator>\n")
    if detectors:
        est += ("    <estimator name=\"reflected\" scores=\"cross\">\n        <surface name=\"p0\"/>\n"
                "    </estimator>\n")
    if detectors is True:
        est += ("    <estimator name=\"interfaces\" scores=\"cross\">\n"
                + "".join(f"        <surface name=\"p{i}\"/>\n" for i in range(n_regions + 1))
                + "    </estimator>\n")
    return _mg_slab_xml(out_dir, "mg_layered_slab", samples, [1.0] * n_regions, tot, sca,
                        [1.0] * n_regions, est)


def _log_uniform_int(rng: np.random.Generator, lo: float, hi: float) -> int:
    """round(exp(U(ln lo, ln hi))) with the exponential in decimal."""
    u = rng.uniform(0.0, 1.0)
    ctx = decimal.Context(prec=40)
    a = ctx.ln(decimal.Decimal(repr(lo)))
    b = ctx.ln(decimal.Decimal(repr(hi)))
    x = ctx.exp(ctx.add(a, ctx.multiply(ctx.subtract(b, a), decimal.Decimal(repr(u)))))
    return int(x.to_integral_value(rounding=decimal.ROUND_HALF_EVEN))


def _mg_sphere_xml(out_dir, name, samples, radii, tot, sca, estimators):
    R, G = tot.shape
    s = [_xml_header(name, samples)]
    s.append(f"<multigroup groups=\"{G}\"/>\n<materials>\n")
    for r in range(R):
        s.append(f"    <material name=\"m{r}\">\n        <multigroup total=\""
                 + " ".join(_fmt(v) for v in tot[r]) + "\"\n            scatter=\""
                 + " ".join(_fmt(v) for v in sca[r].reshape(-1)) + "\"/>\n    </material>\n")
    s.append("</materials>\n<surfaces>\n")
    for i, rad in enumerate(radii):
        s.append(f"    <sphere name=\"s{i}\" x=\"0\" y=\"0\" z=\"0\" r=\"{_fmt(rad)}\"/>\n")
    s.append("</surfaces>\n<cells>\n")
    for r in range(R):
        s.append(f"    <cell name=\"c{r}\" material=\"m{r}\">\n")
        if r > 0:
            s.append(f"        <surface name=\"s{r - 1}\" sense=\"+1\"/>\n")
        s.append(f"        <surface name=\"s{r}\" sense=\"-1\"/>\n    </cell>\n")
    s.append(f"    <cell name=\"outside\" importance=\"0.0\">\n        <surface name=\"s{R - 1}\" sense=\"+1\"/>\n"
             "    </cell>\n</cells>\n")
    s.append("<sources>\n    <point x=\"0\" y=\"0\" z=\"0\" group=\"0\"/>\n</sources>\n")
    s.append("<estimators>\n" + estimators.replace("@R", str(R - 1)) + "</estimators>\n")
    os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(out_dir, "input.xml"), "w") as f:
        f.write("".join(s))
    return out_dir


def batch_shields(root: str, n_problems: int = 4096, min_hist: float = 1e3, max_hist: float = 1e6, k: int = 4):
    """Writes n_problems shield inputs under root/p0000, ... and returns
    [(dir, histories), ...].  Each problem: slab or sphere (p = 1/2), R ~
    U{1..8} regions of equal width, total thickness T ~ U[1, 50] mean free
    paths of the first region's group 1, G = 1 or 8 (p = 1/2), sigma_t,g ~
    U[0.2, 2], scatter ratio ~ U[0.5, 0.95] split downward by Dirichlet(1);
    histories log-uniform on [min_hist, max_hist].  Tally: leakage (slab:
    transmission and reflection) with a group filter."""
    rng = _rng(k)
    out = []
    for i in range(n_problems):
        d = os.path.join(root, f"p{i:04d}")
        sphere = rng.uniform() < 0.5
        R = int(rng.integers(1, 9))
        G = 1 if rng.uniform() < 0.5 else 8
        T = rng.uniform(1.0, 50.0)
        tot, sca = mg_slab_data(R, G, k, rng=rng)
        width = T / tot[0, 0] / R
        n = _log_uniform_int(rng, min_hist, max_hist)
        if sphere:
            radii = [width * (r + 1) for r in range(R)]
            est = ("    <estimator name=\"leakage\" scores=\"cross\">\n        <surface name=\"s@R\"/>\n"
                   "        <filter type=\"group\"/>\n    </estimator>\n")
            _mg_sphere_xml(d, f"sphere{i}", n, radii, tot, sca, est)
        else:
            est = ("    <estimator name=\"leakage\" scores=\"cross\">\n        <surface name=\"p@R\"/>\n"
                   "        <filter type=\"group\"/>\n    </estimator>\n"
                   "    <estimator name=\"reflected\" scores=\"cross\">\n        <surface name=\"p0\"/>\n"
                   "    </estimator>\n")
            _mg_slab_xml(d, f"slab{i}", n, [width] * R, tot, sca, [1.0] * R, est)
        out.append((d, n))
    return out
