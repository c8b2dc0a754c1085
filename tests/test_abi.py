"""The C ABI boundary: the library loads, exports what include/mcgpu.h
declares, and turns input errors into status codes (no GPU needed)."""
import ctypes
import os
import re
import tempfile

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "mcgpu.h")


@pytest.fixture(scope="module")
def L():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "mc-old_gb300"))
    import build as B
    B.build()
    import mcgpu
    return mcgpu.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for need in ("mc_problem_load_xml", "mc_problem_free", "mc_run", "mc_tally_read",
                 "mc_tally_count", "mc_counters_read", "mc_report", "mc_last_error"):
        assert need in names


def test_library_exports_every_declared_symbol(L):
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(L):
    L.mc_status_string.restype = ctypes.c_char_p
    assert L.mc_status_string(0) == b"MC_OK"
    assert L.mc_status_string(4) == b"MC_ERR_LOST"


def _load(L, d):
    h = ctypes.c_void_p()
    st = L.mc_problem_load_xml(os.fsencode(d), os.fsencode(os.path.join(d, "xs_library")), ctypes.byref(h))
    msg = L.mc_last_error(h).decode() if h else ""
    if h:
        L.mc_problem_free(h)
    return st, msg


BAD_INPUTS = {
    "unknown surface type": '<surfaces><torus name="t"/></surfaces>',
    "fission": None,
    "unknown material": '<cells><cell name="c" material="nope"/></cells>',
    "ksearch": '<simulation><description samples="10"/><ksearch active_cycles="1" passive_cycles="1"/></simulation>',
    "comb teeth above bank_max": ('<simulation><description samples="10"/></simulation>'
                                  '<population_control><particle_comb bank_max="5" teeth="10"/></population_control>'),
    "comb without teeth": ('<simulation><description samples="10"/></simulation>'
                           '<population_control><particle_comb bank_max="5"/></population_control>'),
    "unresolved distribution": '<distributions><independentXYZ name="d" datatype="point" x="a" y="b" z="c"/></distributions>',
    "malformed xml": '<surfaces><plane_x name="p" x="1"></surfaces>',
}


@pytest.mark.parametrize("case", list(BAD_INPUTS))
def test_input_errors_are_status_codes(L, case):
    with tempfile.TemporaryDirectory() as d:
        body = BAD_INPUTS[case]
        if case == "fission":
            os.makedirs(os.path.join(d, "xs_library"))
            with open(os.path.join(d, "xs_library", "092235.txt"), "w") as f:
                f.write("235\n0 0\n0 0\n0 0\n1e-5 10 5 100 2.4 0\n2e7 4 0.1 1 2.6 0\n")
            body = '<nuclides><nuclide name="U" ZAID="092235"/></nuclides>'
        with open(os.path.join(d, "input.xml"), "w") as f:
            f.write("<?xml version='1.0'?>\n" + body + "\n")
        st, msg = _load(L, d)
        assert st == 1, (st, msg)   # MC_ERR_INPUT, never an exit
        assert msg
        if case.startswith("comb"):
            assert "particle_comb" in msg, msg


def test_valid_input_parses_before_device_init(L):
    import cases
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        st, msg = _load(L, d)
        # parses; without a GPU the only possible failure is the device
        assert st in (0, 2), (st, msg)
        if st == 2:
            assert "CUDA" in msg or "device" in msg


def test_command_line_driver_usage(L):
    """mcgpu_run (the MC.exe counterpart) is built beside the library and,
    like Main.cpp:11-14, asks for the input directory when given none."""
    import subprocess
    exe = os.path.join(ROOT, "mc-old_gb300", "mcgpu", "mcgpu_run")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Please provide input.xml directory" in r.stdout


def test_command_line_driver_reports_input_errors(L):
    import subprocess
    exe = os.path.join(ROOT, "mc-old_gb300", "mcgpu", "mcgpu_run")
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "input.xml"), "w") as f:
            f.write("<?xml version='1.0'?>\n" + BAD_INPUTS["malformed xml"] + "\n")
        r = subprocess.run([exe, d], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 + 1, r.stdout + r.stderr      # MC_ERR_INPUT, before any device use
    assert "[ERROR] setup" in r.stderr


def test_header_is_plain_c_and_the_ctypes_structs_match_it():
    """include/mcgpu.h compiles as pedantic C99, and the Python layer's
    ctypes copies of mc_tune and mc_counters have the header's size and
    field offsets (a field added on one side only would shift the rest)."""
    import subprocess
    import sys
    sys.path.insert(0, os.path.join(ROOT, "mc-old_gb300"))
    import mcgpu
    structs = {"mc_tune": mcgpu.Tune, "mc_counters": mcgpu.Counters}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "mcgpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as fh:
            fh.write("\n".join(lines) + "\n")
        r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                            "-I", os.path.join(ROOT, "include"), src, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = dict(zip(out[0::2], (int(x) for x in out[1::2])))
    for cname, py in structs.items():
        assert got[cname] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[f"{cname}.{f}"] == getattr(py, f).offset, f"{cname}.{f}"
