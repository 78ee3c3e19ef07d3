"""Build recipe of the C driver (test infrastructure): gcc against the
in-tree libfigpu.so and include/fi_gpu.h, into tests/driver/_build/."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "fi_test_isostasy.c")
OUT = os.path.join(HERE, "_build", "fi_test_isostasy")


def build() -> str:
    from fastisostasy_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT,
           "-L", libdir, "-lfigpu", "-Wl,-rpath," + libdir, "-L", os.path.join(cuda, "lib64"),
           "-Wl,-rpath-link," + os.path.join(cuda, "lib64"), "-lm"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build())
