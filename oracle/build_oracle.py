"""Build recipe for the CPU oracle (test infrastructure).

Compiles ``oracle/fi_oracle.c`` into ``oracle/_build/libfi_oracle.so`` with
OpenMP.  Portable flags only (the same recipe runs on x86_64 and aarch64).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfi_oracle.so")
SRC = os.path.join(HERE, "fi_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(os.path.join(HERE, "fi_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-Wall", "-Wno-unused-variable", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
