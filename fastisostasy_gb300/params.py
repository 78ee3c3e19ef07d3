"""Parameters of the LV-ELVA path: namelist reading and unit handling.

Mirrors ``isos_par_load`` (src/fastisostasy.f90:925-1015) and the
``&barysealevel`` group of ``bsl_init`` (src/barysealevel.f90:40-106): values
are read from a Fortran namelist file and converted the way the reference
converts them (r_earth, pad, zl and dl from km to m).  String options become
the integer codes of the C-ABI (``include/fi_gpu.h``).
"""
from __future__ import annotations

import re

LITHOSPHERE = {"uniform": 0, "gaussian_plus": 1, "gaussian_minus": 2, "rheology_file": 3, "field": 3}
MANTLE = {"uniform": 0, "gaussian_plus": 1, "gaussian_minus": 2, "rheology_file": 3, "field": 3}
LAYERING = {"equalized": 0, "parallel": 1}
LUMPING = {"bottom": 0, "min": 1, "max": 2, "mean": 3, "logmean": 4, "freqdomain": 5}
VISC_SCALING = {"none": 0, "scale": 1, "min": 2, "max": 3, "stddev": 0}
DT_METHOD = {"euler": 0, "rk4": 1, "tsit54": 2}
STAGE_MODE = {"reference": 0, "true": 1}
BSL_METHOD = {"const": 0, "file": 1, "fastiso": 2, "mixed": 3}

# &isostasy of par/test_isostasy_test1d.nml, already in SI units.
DEFAULTS = dict(
    method=3, interactive_sealevel=0, include_elastic=0, heterogeneous_ssh=0,
    correct_compression=0, lithosphere=0, mantle=0, layering=0, lumping=5,
    visc_scaling_method=1, nl=1, dt_method=2, stage_mode=0, nx_target=0, ny_target=0,
    dt_diagnostics=10.0, min_pad=0.0, viscosity_scaling=1.0,
    zl=[88.0e3], viscosities=[1e21], dl=0.0, eta_ref=1e21,
    E=66.0, nu=0.28, rho_water=1000.0, rho_ice=910.0, rho_seawater=1028.0,
    rho_uppermantle=3400.0, rho_litho=0.0, g=9.81, r_earth=6.378e6, m_earth=5.972e24,
    atol=1e-2, rtol=1e-4, dt_min=1e-10, dt_max=10.0, dt_init=1.0, q=1.0,
    tau=3000.0,
)

_CODES = {"lithosphere": LITHOSPHERE, "mantle": MANTLE, "layering": LAYERING, "lumping": LUMPING,
          "viscosity_scaling_method": VISC_SCALING, "dt_method": DT_METHOD}


def _parse_value(tok: str):
    tok = tok.strip()
    if not tok:
        return None
    if tok[0] in "\"'":
        return tok.strip("\"'")
    low = tok.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    if "," in tok:
        return [_parse_value(t) for t in tok.split(",") if t.strip()]
    try:
        if re.fullmatch(r"[+-]?\d+", tok):
            return int(tok)
        return float(tok.lower().replace("d", "e"))
    except ValueError:
        return tok


def read_namelist(text: str, group: str) -> dict:
    """Parse one ``&group ... /`` block of a Fortran namelist (the subset the
    reference's par/*.nml files use: scalars, strings, logicals, lists)."""
    out = {}
    m = re.search(r"&" + re.escape(group) + r"\b(.*?)\n\s*/", text, re.S | re.I)
    if not m:
        raise KeyError("namelist group &%s not found" % group)
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if "=" not in line:
            continue
        key, val = line.split("=", 1)
        out[key.strip()] = _parse_value(val)
    return out


def isostasy_params(nml: dict) -> dict:
    """Convert an ``&isostasy`` group to the flat parameter dict (SI units),
    as isos_par_load does (src/fastisostasy.f90:925-1015)."""
    p = dict(DEFAULTS)
    def as_list(v):
        return list(v) if isinstance(v, list) else [v]
    for k, v in nml.items():
        if k == "pad":
            p["min_pad"] = float(v) * 1e3
        elif k == "r_earth":
            p["r_earth"] = float(v) * 1e3
        elif k == "zl":
            p["zl"] = [float(x) * 1e3 for x in as_list(v)]
        elif k == "dl":
            p["dl"] = float(v) * 1e3
        elif k == "viscosities":
            p["viscosities"] = [float(x) for x in as_list(v)]
        elif k == "ref_viscosity":
            p["eta_ref"] = float(v)
        elif k == "viscosity_scaling_method":
            p["visc_scaling_method"] = VISC_SCALING.get(str(v), 0)
        elif k in _CODES:
            p[k] = _CODES[k][str(v)]
        elif k in ("heterogeneous_ssh", "interactive_sealevel", "include_elastic", "correct_compression"):
            p[k] = int(bool(v))
        elif k in p and not isinstance(v, str):
            p[k] = v
    p["nl"] = int(p["nl"])
    return p


def bsl_params(nml: dict) -> dict:
    return dict(method=BSL_METHOD[str(nml.get("method", "const"))],
                bsl_init=float(nml.get("bsl_init", 0.0)),
                A_ocean_pd=float(nml.get("A_ocean_pd", 3.625e14)))


def load(path: str, group: str = "isostasy") -> dict:
    with open(path) as fh:
        return isostasy_params(read_namelist(fh.read(), group))
