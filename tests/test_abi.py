"""The C-ABI library loads and exports every symbol include/*.h declares."""
import ctypes
import glob
import os
import re

import numpy as np

from conftest import ROOT


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:void\*?|int|long|double)\s*\**\s*(\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return names


def test_exports_match_header(sylver):
    lib = sylver.load()
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert set(sylver.EXPORTS) <= names


LAYOUTS = os.path.join(ROOT, "tests", "golden", "struct_layouts.json")
# our header's name for each reference struct
OURS = {"sylver_inform_t": "sylver_inform_t", "sylver_options_t": "sylver_options_t",
        "options_c": "sylver_options_c", "inform_c": "sylver_inform_c"}


def test_struct_layouts_compiled_against_header(tmp_path):
    """sizeof and offsetof of the four boundary structs, compiled by the C
    compiler against include/sylver_gb300.h, equal the values compiled from
    the reference's own definitions (tests/golden/make_layouts.py)."""
    import json
    import shutil
    import subprocess
    ref = json.load(open(LAYOUTS))
    cc = shutil.which("gcc") or shutil.which("cc")
    assert cc, "no C compiler"
    src = ["#include <stddef.h>", "#include <stdio.h>", '#include "sylver_gb300.h"',
           "int main(void){"]
    for rname, cname in OURS.items():
        src.append(f'printf("{rname} sizeof %zu\\n", sizeof({cname}));')
        for m in ref[rname]:
            if m != "sizeof":
                src.append(f'printf("{rname} {m} %zu\\n", offsetof({cname}, {m}));')
    src.append("return 0;}")
    (tmp_path / "p.c").write_text("\n".join(src) + "\n")
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(tmp_path / "p.c"), "-o",
                    str(tmp_path / "p")], check=True)
    out = subprocess.run([str(tmp_path / "p")], capture_output=True, text=True, check=True)
    got = {}
    for line in out.stdout.splitlines():
        s, m, v = line.split()
        got.setdefault(s, {})[m] = int(v)
    for rname in OURS:
        assert got[rname] == ref[rname], rname


def test_ctypes_mirrors_match_layouts(sylver):
    """The Python binding's Structure mirrors have the same layouts."""
    import json
    ref = json.load(open(LAYOUTS))
    for rname, cls in (("sylver_inform_t", sylver.Inform), ("sylver_options_t", sylver.Options),
                       ("options_c", sylver.OptionsC), ("inform_c", sylver.InformC)):
        assert ctypes.sizeof(cls) == ref[rname]["sizeof"], rname
        for m, off in ref[rname].items():
            if m != "sizeof":
                assert getattr(cls, m).offset == off, (rname, m)


def test_struct_layouts(sylver):
    # option defaults (src/sylver_datatypes_mod.F90:97-198)
    o = sylver.default_options()
    assert o.nemin == 32 and o.nb == 256 and abs(o.u - 0.01) < 1e-15 and o.action
    assert o.ordering == 1 and abs(o.small - 1e-20) < 1e-35


def test_no_gpu_means_error_not_fallback(sylver):
    import torch
    if torch.cuda.is_available():
        return
    from sylver_gb300 import workloads as w
    p = w.laplace2d(6)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val)
    assert f.flag == -51


def test_call_sequence_errors(sylver):
    lib = sylver.load()
    inf = sylver.Inform()
    o = sylver.default_options()
    x = np.zeros(4)
    lib.spldlt_solve(0, 1, x.ctypes.data_as(ctypes.c_void_p), 4, None, None, ctypes.byref(o),
                     ctypes.byref(inf))
    assert inf.flag == -1
    fk = ctypes.c_void_p()
    lib.spldlt_factorize(True, None, None, x.ctypes.data_as(ctypes.c_void_p), None, None,
                         ctypes.byref(fk), ctypes.byref(o), ctypes.byref(inf))
    assert inf.flag == -1


def test_schedule_round_trip(sylver):
    """Every field of sylver_gb300_schedule_t reaches the library and comes
    back; no arguments restore the defaults (zeros)."""
    vals = dict(small_front_rows=96, tc_min_cb_rows=128, solve_large_cols=64, ldlt_tpp_cols=8,
                fs_panel_cols=128, fs_panel_group=3, front_memory=1,
                solve_dataflow=-1)
    try:
        sylver.set_schedule(**vals)
        assert sylver.get_schedule() == vals
    finally:
        sylver.set_schedule()
    assert all(v == 0 for v in sylver.get_schedule().values())
