"""Pin cases: small inputs in the reference's own XML schema.

Each writer fills a directory with input.xml and an xs_library/ of 6-column
tables.  The cases only use schema the reference parses itself
(src/simulator/setup.cpp), so the compiled reference can produce their golden
tallies; together they exercise every hot-path feature the reference has:
planes (axis and general), spheres, cylinders, transmission / reflective /
vacuum boundaries, importance splitting and roulette, weight roulette,
continuous-energy free-gas scatter, uniform and independentXYZ source
distributions, several sources, track-length / collision / crossing
estimators, every non-fission score, energy (grid / lethargy) and time
(grid_linear) filters, and the kernel switch that "cross" applies to the
scores listed after it (setup.cpp:688-690).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "mc-old_gb300"))
from mcgpu import workloads as W  # noqa: E402

SEED = 0x4D43


def _tables(d, specs, n_points=400):
    """specs: list of (zaid, A, s0, Ec, c0); log-uniform grid 1e-5..2e7 eV."""
    os.makedirs(os.path.join(d, "xs_library"), exist_ok=True)
    E = W.log_uniform_grid(1e-5, 2e7, n_points)
    for zaid, A, s0, Ec, c0 in specs:
        W.write_xs_table(os.path.join(d, "xs_library", zaid + ".txt"), A, E,
                         s0 / (1.0 + E / Ec), c0 * np.sqrt(0.0253 / E))


def ce_sphere_small(d, samples=300):
    W.ce_sphere(d, samples=samples, n_points=2000)
    return d


def ce_sphere_bench(d, samples=1000):
    """The benchmark workload itself (continuous-energy three-shell shield,
    20,000-point tables for five nuclides, 50-bin lethargy spectrum) at a
    history count the compiled reference runs in a fraction of a second."""
    W.ce_sphere(d, samples=samples, n_points=20_000)
    return d


def slab_features(d, samples=400):
    _tables(d, [("700001", 1.0, 6.0, 1e6, 0.3), ("700016", 16.0, 4.0, 3e6, 0.05),
                ("700012", 12.0, 5.0, 2e6, 0.01)])
    xml = """<?xml version = '1.0' encoding = 'UTF-8'?>
<simulation>
    <description name="slab features" samples="%d"/>
</simulation>
<nuclides>
    <nuclide name="H" ZAID="700001"/>
    <nuclide name="O" ZAID="700016"/>
    <nuclide name="C" ZAID="700012"/>
</nuclides>
<materials>
    <material name="water"><nuclide name="H" density="0.06"/><nuclide name="O" density="0.03"/></material>
    <material name="carbon"><nuclide name="C" density="0.09"/></material>
</materials>
<surfaces>
    <plane_x name="x0" x="0.0"/>
    <plane_x name="x1" x="2.0"/>
    <plane_x name="x2" x="4.0"/>
    <plane_x name="x3" x="6.0"/>
    <plane_x name="x4" x="8.0"/>
    <plane_x name="x5" x="10.0"/>
    <plane_y name="ylo" y="-3.0" bc="reflective"/>
    <plane_y name="yhi" y="3.0" bc="reflective"/>
    <plane_z name="zlo" z="-4.0" bc="vacuum"/>
    <plane_z name="zhi" z="4.0" bc="vacuum"/>
</surfaces>
<cells>
    <cell name="r0" material="water" importance="1.0">
        <surface name="x0" sense="+1"/><surface name="x1" sense="-1"/>
        <surface name="ylo" sense="+1"/><surface name="yhi" sense="-1"/>
        <surface name="zlo" sense="+1"/><surface name="zhi" sense="-1"/>
    </cell>
    <cell name="r1" material="carbon" importance="2.0">
        <surface name="x1" sense="+1"/><surface name="x2" sense="-1"/>
        <surface name="ylo" sense="+1"/><surface name="yhi" sense="-1"/>
        <surface name="zlo" sense="+1"/><surface name="zhi" sense="-1"/>
    </cell>
    <cell name="r2" material="water" importance="4.0">
        <surface name="x2" sense="+1"/><surface name="x3" sense="-1"/>
        <surface name="ylo" sense="+1"/><surface name="yhi" sense="-1"/>
        <surface name="zlo" sense="+1"/><surface name="zhi" sense="-1"/>
    </cell>
    <cell name="r3" importance="2.5">
        <surface name="x3" sense="+1"/><surface name="x4" sense="-1"/>
        <surface name="ylo" sense="+1"/><surface name="yhi" sense="-1"/>
        <surface name="zlo" sense="+1"/><surface name="zhi" sense="-1"/>
    </cell>
    <cell name="r4" material="carbon" importance="1.0">
        <surface name="x4" sense="+1"/><surface name="x5" sense="-1"/>
        <surface name="ylo" sense="+1"/><surface name="yhi" sense="-1"/>
        <surface name="zlo" sense="+1"/><surface name="zhi" sense="-1"/>
    </cell>
    <cell name="left" importance="0.0"><surface name="x0" sense="-1"/></cell>
    <cell name="right" importance="0.0"><surface name="x5" sense="+1"/></cell>
</cells>
<distributions>
    <uniform name="Eu" datatype="double" a="1e5" b="2e6"/>
    <uniform name="ux" datatype="double" a="0.3" b="1.0"/>
    <uniform name="uy" datatype="double" a="-0.4" b="0.4"/>
    <delta name="uz" datatype="double" val="0.1"/>
    <independentXYZ name="beam" datatype="point" x="ux" y="uy" z="uz"/>
    <isotropic name="iso" datatype="point"/>
    <delta name="E1" datatype="double" val="1.5e6"/>
</distributions>
<sources>
    <point x="1e-6" y="0.5" z="-0.25" direction="beam" energy="Eu"/>
    <point x="1.0" y="0.0" z="0.0" direction="iso" energy="E1"/>
    <point x="5.0" y="-1.0" z="1.0" energy="Eu"/>
</sources>
<estimators>
    <estimator name="tl_all" scores="flux absorption scatter capture total">
        <cell name="r0"/><cell name="r1"/><cell name="r2"/><cell name="r4"/>
        <filter type="energy" grid="1e-5 1.0 1e3 1e5 1e6 2e7"/>
    </estimator>
    <estimator name="tl_time" scores="flux">
        <cell name="r1"/><cell name="r2"/><cell name="r3"/>
        <filter type="time" grid_linear="0.0 2e-9 2e-8"/>
    </estimator>
    <estimator name="coll" type="C" scores="flux total capture">
        <cell name="r0"/><cell name="r2"/><cell name="r4"/>
    </estimator>
    <estimator name="leak" scores="cross">
        <surface name="x0"/><surface name="x5"/>
        <filter type="energy" grid_lethargy="1e-5 2e7 8"/>
    </estimator>
    <estimator name="cross_then_flux" scores="cross flux">
        <surface name="x3"/><surface name="zhi"/>
    </estimator>
    <estimator name="crossing_time" scores="cross">
        <surface name="x2"/>
        <filter type="time" grid="0 1e-9 3e-9 1e-8 1e-7"/>
    </estimator>
</estimators>
""" % samples
    with open(os.path.join(d, "input.xml"), "w") as f:
        f.write(xml)
    return d


def quadrics(d, samples=300):
    _tables(d, [("710001", 1.0, 8.0, 1e6, 0.2), ("710012", 12.0, 5.0, 2e6, 0.02)])
    xml = """<?xml version = '1.0' encoding = 'UTF-8'?>
<simulation>
    <description name="quadrics" samples="%d"/>
</simulation>
<nuclides>
    <nuclide name="H" ZAID="710001"/>
    <nuclide name="C" ZAID="710012"/>
</nuclides>
<materials>
    <material name="mod"><nuclide name="H" density="0.05"/><nuclide name="C" density="0.02"/></material>
    <material name="gr"><nuclide name="C" density="0.08"/></material>
</materials>
<surfaces>
    <cylinder_z name="cz" x="0.5" y="-0.5" r="3.0"/>
    <cylinder_x name="cx" y="0.0" z="0.0" r="8.0"/>
    <plane name="tilt" a="1.0" b="0.5" c="-0.25" d="6.0" bc="reflective"/>
    <plane name="back" a="-1.0" b="0.2" c="0.1" d="6.0"/>
    <sphere name="ball" x="0.0" y="1.0" z="0.0" r="1.5"/>
</surfaces>
<cells>
    <cell name="ballc" material="gr" importance="1.0">
        <surface name="ball" sense="-1"/>
    </cell>
    <cell name="core" material="mod">
        <surface name="ball" sense="+1"/><surface name="cz" sense="-1"/>
        <surface name="tilt" sense="-1"/><surface name="back" sense="-1"/>
    </cell>
    <cell name="annulus" material="gr" importance="0.5">
        <surface name="cz" sense="+1"/><surface name="cx" sense="-1"/>
        <surface name="tilt" sense="-1"/><surface name="back" sense="-1"/>
    </cell>
    <cell name="outside" importance="0.0">
        <surface name="cx" sense="+1"/><surface name="tilt" sense="-1"/><surface name="back" sense="-1"/>
    </cell>
    <cell name="beyond" importance="0.0"><surface name="back" sense="+1"/></cell>
</cells>
<sources>
    <point x="0.0" y="-1.0" z="0.5"/>
</sources>
<estimators>
    <estimator name="cells" scores="flux total">
        <cell name="ballc"/><cell name="core"/><cell name="annulus"/>
    </estimator>
    <estimator name="coll" type="C" scores="absorption scatter">
        <cell name="core"/><cell name="annulus"/>
        <filter type="energy" grid_lethargy="1e-5 2e7 5"/>
    </estimator>
    <estimator name="out" scores="cross">
        <surface name="cx"/><surface name="back"/>
    </estimator>
    <estimator name="refl" scores="cross">
        <surface name="tilt"/>
    </estimator>
</estimators>
""" % samples
    with open(os.path.join(d, "input.xml"), "w") as f:
        f.write(xml)
    return d


def absorber_slab(d, samples=100_000):
    """The reference's examples/slab_analytic problem (leakage e^-4.2 =
    0.0149956, test/test_integral_Simulator.cpp:20-29) with its three
    capture-only nuclides written as constant 2-point tables, the form the
    reference can run (its user-defined nuclides leave sigma_t unset)."""
    os.makedirs(os.path.join(d, "xs_library"), exist_ok=True)
    for zaid, c in (("720001", 1.0), ("720002", 0.5), ("720003", 2.0)):
        W.write_xs_table(os.path.join(d, "xs_library", zaid + ".txt"), 1.0, [1e-5, 2e7],
                         [0.0, 0.0], [c, c])
    xml = """<?xml version = '1.0' encoding = 'UTF-8'?>
<simulation>
    <description name="Simple Slabs" samples="%d"/>
</simulation>
<nuclides>
    <nuclide name="nuc1" ZAID="720001"/>
    <nuclide name="nuc2" ZAID="720002"/>
    <nuclide name="nuc3" ZAID="720003"/>
</nuclides>
<materials>
    <material name="mat1">
        <nuclide name="nuc1" density="0.5"/><nuclide name="nuc2" density="1.0"/><nuclide name="nuc3" density="0.1"/>
    </material>
    <material name="mat2">
        <nuclide name="nuc1" density="0.5"/><nuclide name="nuc2" density="0.5"/>
    </material>
</materials>
<surfaces>
    <plane_x name="px1" x="0.0"/>
    <plane_x name="px2" x="1.0"/>
    <plane_x name="px3" x="5.0"/>
</surfaces>
<cells>
    <cell name="slab1" material="mat1"><surface name="px1" sense="+1"/><surface name="px2" sense="-1"/></cell>
    <cell name="slab2" material="mat2"><surface name="px2" sense="+1"/><surface name="px3" sense="-1"/></cell>
    <cell name="left outside" importance="0.0"><surface name="px1" sense="-1"/></cell>
    <cell name="right outside" importance="0.0"><surface name="px3" sense="+1"/></cell>
</cells>
<distributions>
    <delta name="dir" datatype="point" x = "1.0" y = "0.0" z = "0.0"/>
</distributions>
<sources>
    <point x="1e-9" y="0.0" z="0.0" direction="dir"/>
</sources>
<estimators>
    <estimator name="leak_rate" scores="cross">
        <surface name="px3"/>
    </estimator>
</estimators>
""" % samples
    with open(os.path.join(d, "input.xml"), "w") as f:
        f.write(xml)
    return d


def absorber_slab_user_nuclides(d, samples=100_000):
    """examples/slab_analytic/input.xml as the reference ships it: user-defined
    capture-only nuclides (the reference itself crashes on it; the oracle and
    the GPU path give these nuclides sigma_t = sigma_c)."""
    xml = """<?xml version = '1.0' encoding = 'UTF-8'?>
<simulation>
    <description name="Simple Slabs" samples="%d"/>
</simulation>
<nuclides>
    <nuclide name="nuc1"><capture xs="1.0"/></nuclide>
    <nuclide name="nuc2"><capture xs="0.5"/></nuclide>
    <nuclide name="nuc3"><capture xs="2.0"/></nuclide>
</nuclides>
<materials>
    <material name="mat1">
        <nuclide name="nuc1" density="0.5"/><nuclide name="nuc2" density="1.0"/><nuclide name="nuc3" density="0.1"/>
    </material>
    <material name="mat2"><nuclide name="nuc1" density="0.5"/><nuclide name="nuc2" density="0.5"/></material>
</materials>
<surfaces>
    <plane_x name="px1" x="0.0"/>
    <plane_x name="px2" x="1.0"/>
    <plane_x name="px3" x="5.0"/>
</surfaces>
<cells>
    <cell name="slab1" material="mat1"><surface name="px1" sense="+1"/><surface name="px2" sense="-1"/></cell>
    <cell name="slab2" material="mat2"><surface name="px2" sense="+1"/><surface name="px3" sense="-1"/></cell>
    <cell name="left outside" importance="0.0"><surface name="px1" sense="-1"/></cell>
    <cell name="right outside" importance="0.0"><surface name="px3" sense="+1"/></cell>
</cells>
<distributions>
    <delta name="dir" datatype="point" x = "1.0" y = "0.0" z = "0.0"/>
</distributions>
<sources>
    <point x="1e-9" y="0.0" z="0.0" direction="dir"/>
</sources>
<estimators>
    <estimator name="leak_rate" scores="cross">
        <surface name="px3"/>
    </estimator>
</estimators>
""" % samples
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "input.xml"), "w") as f:
        f.write(xml)
    return d


def comb_slab(d, samples=300, bank_max=3, teeth=2):
    """slab_features with steep importances (1, 3, 9, 4, 2) and the particle
    comb (population_control.cpp:55-84): banks of split copies reach
    bank_max often, so the comb acts many times per history."""
    slab_features(d, samples)
    path = os.path.join(d, "input.xml")
    with open(path) as f:
        xml = f.read()
    for name, old, new in [("r1", "2.0", "3.0"), ("r2", "4.0", "9.0"), ("r3", "2.5", "4.0"), ("r4", "1.0", "2.0")]:
        a = '<cell name="%s" material' % name if name != "r3" else '<cell name="%s" importance' % name
        i = xml.index(a)
        j = xml.index('importance="%s"' % old, i)
        xml = xml[:j] + 'importance="%s"' % new + xml[j + len('importance="%s"' % old):]
    xml = xml.replace("</simulation>\n", "</simulation>\n<population_control>\n"
                      '    <particle_comb bank_max="%d" teeth="%d"/>\n</population_control>\n' % (bank_max, teeth), 1)
    with open(path, "w") as f:
        f.write(xml)
    return d


# cases the compiled reference can run, with their golden-file names
REFERENCE_CASES = {
    "ce_sphere_small": ce_sphere_small,
    "ce_sphere_bench": ce_sphere_bench,
    "slab_features": slab_features,
    "quadrics": quadrics,
    "absorber_slab": absorber_slab,
    "comb_slab": comb_slab,
}


def write_case(name: str, d: str) -> str:
    os.makedirs(d, exist_ok=True)
    return REFERENCE_CASES[name](d)
