"""CPU tests: the C-ABI library builds and exports every declared symbol;
host-side parameter handling; workload generators.  No GPU calls."""
import ctypes
import os
import re
import subprocess

import numpy as np

from fastisostasy_gb300 import build as B
from fastisostasy_gb300 import params as P
from fastisostasy_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            syms |= set(re.findall(r"\b(fi_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_exports_all_declared_symbols():
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing
    assert len(declared_symbols()) >= 20


def test_c_abi_struct_layout_matches_binding(tmp_path):
    """The ctypes structs match the C header's layout (compiled with gcc)."""
    from fastisostasy_gb300._lib import FiBsl, FiOut, FiParams
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "fi_gpu.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(fi_params), sizeof(fi_bsl),'
                   ' sizeof(fi_out), offsetof(fi_params, dt_diagnostics), offsetof(fi_params, q),'
                   ' offsetof(fi_bsl, series_t)); return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(FiParams), ctypes.sizeof(FiBsl), ctypes.sizeof(FiOut),
            FiParams.dt_diagnostics.offset, FiParams.q.offset, FiBsl.series_t.offset]
    assert got == want


def test_namelist_parser_units():
    text = """
&isostasy
    include_elastic = .true.   ! comment
    pad = 512.
    zl = 70., 600.
    viscosities = 1.e21, 4.e21
    lumping = "freqdomain"
    dt_method = "rk4"
    r_earth = 6.378e3
/
"""
    p = P.isostasy_params(P.read_namelist(text, "isostasy"))
    assert p["include_elastic"] == 1 and p["min_pad"] == 512e3
    assert p["zl"] == [70e3, 600e3] and p["viscosities"] == [1e21, 4e21]
    assert p["lumping"] == 5 and p["dt_method"] == 1 and p["r_earth"] == 6.378e6


def test_workloads_are_seeded():
    a = W.config3(nx_ice=48, ny_ice=80, nx_pad=64, ny_pad=96)
    b = W.config3(nx_ice=48, ny_ice=80, nx_pad=64, ny_pad=96)
    assert np.array_equal(a.z_bed, b.z_bed) and np.array_equal(a.H_final, b.H_final)
    m0, m1 = W.ensemble_member(0), W.ensemble_member(0)
    assert m0.nx_ice == m1.nx_ice and m0.dx == m1.dx
    f0 = m0.padded_fields(m0.nx_ice, m0.ny_ice)["eta_eff"]
    f1 = m1.padded_fields(m1.nx_ice, m1.ny_ice)["eta_eff"]
    assert np.array_equal(f0, f1)
    assert abs(np.log10(f0).mean() - 21.0) < 1e-9


def _header_functions():
    """{name: number of parameters} of every function fi_gpu.h declares."""
    text = open(os.path.join(ROOT, "include", "fi_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(fi_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def _fortran_interfaces():
    """{C name: number of dummy arguments} of the interface blocks in
    include/fastisostasy_gpu.f90, and the components of its bind(C) types."""
    text = open(os.path.join(ROOT, "include", "fastisostasy_gpu.f90")).read()
    text = re.sub(r"!.*", "", text).replace("&\n", " ")
    funcs = {}
    for m in re.finditer(r"function[ \t]+(\w+)[ \t]*\(([^)]*)\)[^\n]*bind\(C,\s*name=\"(\w+)\"\)", text, re.I):
        args = [a for a in m.group(2).replace(" ", "").split(",") if a]
        assert m.group(1) == m.group(3)
        funcs[m.group(3)] = len(args)
    types = {}
    for m in re.finditer(r"type,\s*bind\(C\)\s*::\s*(\w+)(.*?)end type", text, re.S | re.I):
        comps = []
        for line in m.group(2).splitlines():
            if "::" in line:
                for c in line.split("::", 1)[1].split(","):
                    c = re.sub(r"\(.*", "", c.strip())
                    if c:
                        comps.append(c.lower())
        types[m.group(1)] = comps
    return funcs, types


def test_fortran_module_binds_every_entry_point():
    """No Fortran compiler exists here: the interface module is checked
    against the header instead.  Every function of fi_gpu.h has an
    interface of the same name and arity, and the bind(C) types list the
    C structs' fields in the same order as the ctypes mirror (whose layout
    the gcc test above checks)."""
    from fastisostasy_gb300 import _lib as L
    hdr = _header_functions()
    funcs, types = _fortran_interfaces()
    assert set(funcs) == set(hdr), (set(hdr) ^ set(funcs))
    for name, n in hdr.items():
        assert funcs[name] == n, (name, funcs[name], n)
    for ftype, ctype in (("fi_params", L.FiParams), ("fi_bsl", L.FiBsl), ("fi_out", L.FiOut),
                         ("fi_rheology", L.FiRheology), ("fi_request", L.FiRequest),
                         ("fi_request_info", L.FiRequestInfo)):
        assert types[ftype] == [f[0].lower() for f in ctype._fields_], ftype


def test_c_driver_builds_and_fails_loudly_without_a_gpu(tmp_path):
    """The C driver that replays the reference's test loop compiles and
    links against libfigpu.so; without a GPU its isos_init fails with
    FI_E_CUDA (there is no CPU path)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "driver"))
    import build_driver
    exe = build_driver.build()
    r = subprocess.run([exe, str(tmp_path / "o.bin"), "0", "33", "100e3", "3", "10", "10"], capture_output=True,
                       text=True)
    assert r.returncode == 6, (r.returncode, r.stderr)
    assert "isos_init" in r.stderr
