"""Regenerates the golden fixtures in this folder.

1. params_<test>.json: the reference's experiment namelists
   (par/test_isostasy_<test>.nml of the reference project) parsed with
   fastisostasy_gb300.params, kei_reference.npz: the reference's
   Kelvin-function table, and ge_reference.npz: its elastic Green's-function
   table — these need the reference tree, so they are only
   made where that tree is mounted (pass its path as argv[1]).
2. oracle_golden.npz: outputs of the cases in tests/make_golden_cases.py.

Usage: python tests/golden/make_golden.py [path/to/reference]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.dirname(HERE)]

import numpy as np  # noqa: E402

from fastisostasy_gb300 import params as P  # noqa: E402

TESTS = ["test1a", "test1b", "test1c", "test1d", "test1e", "test2a", "test2b", "test2c", "test3a", "test3b",
         "test3c", "test3d"]


def kei_reference(ref):
    """The reference's tabulated Kelvin function kei (load_kei_values in
    src/kelvin_function.f90), read from its source: 1001 (x, kei) pairs
    written as default-real literals, hence rounded to single precision."""
    import re
    with open(os.path.join(ref, "src", "kelvin_function.f90")) as fh:
        src = fh.read()
    blk = src[src.index("tbl = ["):]
    blk = blk[:blk.index("]")]
    nums = [float(x) for x in re.findall(r"[-+]?\d+\.\d+(?:E[-+]\d+)?", blk)]
    t = np.array(nums, dtype=np.float32).astype(np.float64).reshape(-1, 2)
    return t[:, 0], t[:, 1]


def ge_reference(ref):
    """The reference's Farrell elastic Green's-function table
    (calc_elastic_green, src/green_functions.f90: rn_vals, ge_vals), read
    from its source: 42 radii [km] and values, default-real literals hence
    single precision; the radii are scaled by 1.e3 in single precision."""
    import re
    with open(os.path.join(ref, "src", "green_functions.f90")) as fh:
        src = fh.read()

    def table(name):
        blk = src[src.index(name):]
        blk = blk[blk.index("[") + 1:blk.index("]")]
        return np.array([float(x) for x in re.findall(r"[-+]?\d+\.\d*", blk)], dtype=np.float32)
    rn = (table("rn_vals") * np.float32(1.e3)).astype(np.float64)
    ge = table("ge_vals").astype(np.float64)
    return rn, ge


def main():
    if len(sys.argv) > 1:
        ref = sys.argv[1]
        for t in TESTS:
            path = os.path.join(ref, "par", "test_isostasy_%s.nml" % t)
            p = P.load(path)
            with open(os.path.join(HERE, "params_%s.json" % t), "w") as fh:
                json.dump(p, fh, indent=1, sort_keys=True)
        rn, kei = kei_reference(ref)
        np.savez_compressed(os.path.join(HERE, "kei_reference.npz"), rn=rn, kei=kei)
        rn, ge = ge_reference(ref)
        assert len(rn) == 42 and len(ge) == 42
        np.savez_compressed(os.path.join(HERE, "ge_reference.npz"), rn=rn, ge=ge)
    import make_golden_cases as MG
    out = {}
    for name, fn in MG.CASES.items():
        for k, v in fn().items():
            out[name + "__" + k] = v
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
