"""Build recipe for the CPU oracle library (test infrastructure only).

Compiles ``oracle/sdemc_oracle.c`` with gcc into ``oracle/_build/libsdemc_oracle.so``.
``-ffp-contract=off`` keeps every float operation separately rounded, so the
oracle reproduces the GPU kernels' explicit operation order bit for bit.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsdemc_oracle.so")
SRC = os.path.join(HERE, "sdemc_oracle.c")


def build():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-pthread", SRC, "-o", tmp, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
